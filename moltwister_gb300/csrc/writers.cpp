// Trajectory writers of the `moldyn run` output step, host code: the DCD records of
// CDCDFile::createDCDFileIfNotExists / appendToDCDFile (Utilities/DCDFile.cpp:137-230, 275-302,
// 403-465, 670-729) as CMDLoop::appendToDCDFile calls them (MDLoop.cpp:248-258), and the XYZ frames
// of CMDLoop::appendToXYZFile (MDLoop.cpp:229-246).  The byte layout is the reference's, so that
// its readers (and VMD) read these files.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/mtgpu.h"

namespace {

bool put(FILE* f, const void* p, size_t n) { return fwrite(p, 1, n, f) == n; }
bool put_u32(FILE* f, uint32_t v) { return put(f, &v, 4); }

// CHARMM-style main header: 84-byte block (ID, sets, first step, stride, 6 zeros, time step,
// 1, 8 zeros, 1), 164-byte title block of two 80-character lines, 4-byte atom count block.
bool dcd_header(FILE* f, uint32_t nsets, uint32_t stride, float timestep, uint32_t natoms) {
    bool ok = put_u32(f, 84) && put(f, "CORD", 4) && put_u32(f, nsets) && put_u32(f, 0) && put_u32(f, stride);
    for(int i = 0; i < 6; i++) ok = ok && put_u32(f, 0);
    ok = ok && put(f, &timestep, 4);
    const uint32_t tail[13] = {1, 0, 0, 0, 0, 0, 0, 0, 0, 1, 84, 164, 2};
    for(uint32_t v : tail) ok = ok && put_u32(f, v);
    char title[80];
    std::memset(title, 0, sizeof title);
    std::memcpy(title, "Written by MolTwister", 21);
    ok = ok && put(f, title, 80);
    std::memset(title, 0, sizeof title);
    std::memcpy(title, "---", 3);
    ok = ok && put(f, title, 80);
    ok = ok && put_u32(f, 164) && put_u32(f, 4) && put_u32(f, natoms) && put_u32(f, 4);
    return ok;
}

}  // namespace

extern "C" {

int mtg_dcd_append(const char* path, int32_t n_atoms, const double* r, const double box[3], int32_t num_steps,
                   int32_t out_stride, double timestep_fs) {
    if(!path || n_atoms <= 0 || !r || !box || out_stride <= 0) return MTG_E_INVALID;
    FILE* f = std::fopen(path, "r");
    if(!f) {
        f = std::fopen(path, "w");
        if(!f) return MTG_E_INVALID;
        const bool ok = dcd_header(f, (uint32_t)(num_steps / out_stride), (uint32_t)out_stride, (float)timestep_fs,
                                   (uint32_t)n_atoms);
        std::fclose(f);
        if(!ok) return MTG_E_INVALID;
    } else {
        std::fclose(f);
    }
    f = std::fopen(path, "a+");
    if(!f) return MTG_E_INVALID;
    // record header: 48-byte block of six doubles (box x, angle, box y, angle, angle, box z); the
    // box arrives as integers (MDLoop.cpp:257 passes it through std::tuple<int, int, int>)
    const double cell[6] = {(double)(int)box[0], 0.0, (double)(int)box[1], 0.0, 0.0, (double)(int)box[2]};
    bool ok = put_u32(f, 48) && put(f, cell, 48) && put_u32(f, 48);
    std::vector<float> c((size_t)n_atoms);
    const uint32_t bytes = (uint32_t)(n_atoms * sizeof(float));
    for(int a = 0; a < 3 && ok; a++) {
        for(int i = 0; i < n_atoms; i++) c[i] = (float)r[3 * i + a];
        ok = put_u32(f, bytes) && put(f, c.data(), bytes) && put_u32(f, bytes);
    }
    std::fclose(f);
    return ok ? MTG_OK : MTG_E_INVALID;
}

int mtg_xyz_append(const char* path, int32_t n_atoms, const double* r, const char* const* ids, int32_t step) {
    if(!path || n_atoms <= 0 || !r || !ids) return MTG_E_INVALID;
    FILE* f = std::fopen(path, "a+");
    if(!f) return MTG_E_INVALID;
    std::fprintf(f, "%i\r\nFrame %u\r\n", (int)n_atoms, (unsigned)step);
    for(int k = 0; k < n_atoms; k++)
        std::fprintf(f, "%-15s% -15g%-15g%-15g\r\n", ids[k], r[3 * k], r[3 * k + 1], r[3 * k + 2]);
    std::fclose(f);
    return MTG_OK;
}

}  // extern "C"
