// Reference-mode kernels: MolTwister's MD arithmetic reproduced on the GPU.
//
// These kernels replace the Thrust functors and serial kernels of the reference
// (FunctorGenCellList.cpp:49-142, FunctorGenNeighList.cpp:72-191, FunctorCalcForce.cpp:95-709) and the
// host loops of VelVerlet.cpp:74-122 / SimulationBox.cpp:135-166 in the parity mode.  The cell
// assignment, neighbour order and per-atom summation order are the reference's, and this file is
// compiled with -fmad=false so no multiply-add is fused: cell lists and neighbour lists are
// bit-identical to the reference and per-atom forces agree to the last few ulps (libm acos may
// differ in the last bit).
//
// Parallel structure: one thread per atom for the gather kernels (the reference's per-atom order
// is sequential), a counting sort with a per-cell rank pass for the cell list (the reference's
// serial kernelAssembleList order is ascending atom index within each cell), and grid-wide
// deterministic reductions for the kinetic energy with the thermostat in the last block.
#include <float.h>
#include <stdint.h>

#include "md_device.cuh"
#include "mtg_internal.h"

namespace mtg {
namespace {

struct D3 {
    double x, y, z;
};
__device__ __forceinline__ D3 d3(double x, double y, double z) { return {x, y, z}; }
__device__ __forceinline__ D3 sub(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 scl(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ double dotp(D3 a, D3 b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); }
__device__ __forceinline__ double nrm(D3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
__device__ __forceinline__ D3 crs(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ D3 load3(const double* r, int i) { return {r[3 * i], r[3 * i + 1], r[3 * i + 2]}; }

// C3DVector::moveToSameSideOfPBCAsThis (Utilities/3DVector.cpp:133-165)
__device__ __forceinline__ void same_side(D3 c, D3& v, const double* w) {
    double dX = c.x - v.x, dY = c.y - v.y, dZ = c.z - v.z;
    dX = (dX < 0.0) ? -dX : dX;
    dY = (dY < 0.0) ? -dY : dY;
    dZ = (dZ < 0.0) ? -dZ : dZ;
    if(dX > (w[0] / 2.0)) { if(c.x > v.x) v.x += w[0]; else v.x -= w[0]; }
    if(dY > (w[1] / 2.0)) { if(c.y > v.y) v.y += w[1]; else v.y -= w[1]; }
    if(dZ > (w[2] / 2.0)) { if(c.z > v.z) v.z += w[2]; else v.z -= w[2]; }
}

__device__ D3 coeff12(D3 r1, D3 r2) {
    D3 r12 = sub(r2, r1);
    double R = nrm(r12);
    return scl(r12, (R == 0.0) ? 1.0 / 1E-10 : 1.0 / R);
}

__device__ D3 coeff_ang13(D3 r1, D3 r2, D3 r3) {
    D3 r12 = sub(r1, r2);
    double R = nrm(r12);
    D3 K = scl(r12, (R == 0.0) ? 1.0 / 1E-10 : 1.0 / R);
    D3 r32 = sub(r3, r2);
    double A = K.x * r32.x + K.y * r32.y + K.z * r32.z;
    double B = r32.x * r32.x + r32.y * r32.y + r32.z * r32.z;
    double sB = sqrt(B);
    double sB3 = (B == 0.0) ? sqrt(1E-30) : sB * sB * sB;
    double gx = (K.x * B - r32.x * A) / sB3, gy = (K.y * B - r32.y * A) / sB3, gz = (K.z * B - r32.z * A) / sB3;
    double W = (sB == 0.0) ? A / 10E-3 : A / sB;
    double den = sqrt(1.0 - W * W);
    double f = (den == 0.0) ? -1.0 / 1E-10 : -1.0 / den;
    return {f * gx, f * gy, f * gz};
}

__device__ D3 coeff_ang2(D3 r1, D3 r2, D3 r3) {
    D3 r12 = sub(r1, r2), r32 = sub(r3, r2);
    double A = r12.x * r12.x + r12.y * r12.y + r12.z * r12.z;
    double B = r32.x * r32.x + r32.y * r32.y + r32.z * r32.z;
    double C = r12.x * r32.x + r12.y * r32.y + r12.z * r32.z;
    double AB = A * B;
    double sAB = sqrt(AB);
    double sAB3 = (AB == 0.0) ? sqrt(1E-30) : sAB * sAB * sAB;
    double gx = ((2.0 * r2.x - r1.x - r3.x) * AB + (r32.x * A + r12.x * B) * C) / sAB3;
    double gy = ((2.0 * r2.y - r1.y - r3.y) * AB + (r32.y * A + r12.y * B) * C) / sAB3;
    double gz = ((2.0 * r2.z - r1.z - r3.z) * AB + (r32.z * A + r12.z * B) * C) / sAB3;
    double W = (sAB == 0.0) ? A / 10E-3 : C / sAB;
    double den = sqrt(1.0 - W * W);
    double f = (den == 0.0) ? -1.0 / 1E-10 : -1.0 / den;
    return {f * gx, f * gy, f * gz};
}

__device__ D3 coeff_dih14(D3 r1, D3 r2, D3 r3, D3 r4) {
    D3 r21 = sub(r1, r2), r23 = sub(r3, r2);
    D3 r32 = scl(r23, -1.0);
    D3 r34 = sub(r4, r3);
    D3 n1 = crs(r23, r21);
    double n1n = nrm(n1);
    D3 K = scl(n1, (n1n == 0.0) ? 1.0 / 1E-10 : 1.0 / n1n);
    double a = r32.y * r34.z - r32.z * r34.y;
    double b = r32.z * r34.x - r32.x * r34.z;
    double c = r32.x * r34.y - r32.y * r34.x;
    double A = K.x * a + K.y * b + K.z * c;
    double B = a * a + b * b + c * c;
    double sBi = (B == 0.0) ? 1.0 / 1E-20 : 1.0 / sqrt(B);
    double sBi3 = sBi * sBi * sBi;
    double W = A * sBi;
    double gx = ((K.y * r32.z - K.z * r32.y) * B - (r32.z * (r32.z * r34.x - r32.x * r34.z) - r32.y * (r32.x * r34.y - r32.y * r34.x)) * A) * sBi3;
    double gy = ((K.z * r32.x - K.x * r32.z) * B - (r32.x * (r32.x * r34.y - r32.y * r34.x) - r32.z * (r32.y * r34.z - r32.z * r34.y)) * A) * sBi3;
    double gz = ((K.x * r32.y - K.y * r32.x) * B - (r32.y * (r32.y * r34.z - r32.z * r34.y) - r32.x * (r32.z * r34.x - r32.x * r34.z)) * A) * sBi3;
    double den = sqrt(1.0 - W * W);
    double f = (den == 0.0) ? 1.0 / 1E-10 : 1.0 / den;
    return scl(d3(f * gx, f * gy, f * gz), -1.0);
}

__device__ D3 coeff_dih23(D3 r1, D3 r2, D3 r3, D3 r4) {
    D3 r21 = sub(r1, r2), r23 = sub(r3, r2);
    D3 r32 = scl(r23, -1.0);
    D3 r34 = sub(r4, r3);
    double K1 = r32.z * r34.x - r32.x * r34.z, K2 = r34.z - r32.z, K3 = r23.z * r21.x - r23.x * r21.z;
    double K4 = r32.x * r34.y - r32.y * r34.x, K5 = r32.y - r34.y, K6 = r23.x * r21.y - r23.y * r21.x;
    double L1 = r32.y * r34.z - r32.z * r34.y, L2 = -K2, L3 = r23.y * r21.z - r23.z * r21.y;
    double L4 = K4, L5 = r34.x - r32.x, L6 = K6;
    double M1 = L1, M2 = -K5, M3 = L3, M4 = K1, M5 = -L5, M6 = K3;
    double A = L3 * L3 + K3 * K3 + K6 * K6;
    double B = L1 * L1 + K1 * K1 + K4 * K4;
    double C = L3 * L1 + K3 * K1 + K6 * K4;
    double AB = A * B;
    double sABi = (AB == 0.0) ? 1.0 / 1E-20 : 1.0 / sqrt(AB);
    double sABi3 = sABi * sABi * sABi;
    double W = C * sABi;
    double dCx = K2 * K3 + r21.y * K4 + K5 * K6 - r21.z * K1;
    double dCy = L2 * L3 - r21.x * L4 + L5 * L6 + r21.z * L1;
    double dCz = M2 * M3 + r21.x * M4 + M5 * M6 - r21.y * M1;
    double gx = (dCx * AB - C * ((r21.y * K6 - r21.z * K3) * B + (K1 * K2 + K4 * K5) * A)) * sABi3;
    double gy = (dCy * AB - C * ((r21.z * L3 - r21.x * L6) * B + (L1 * L2 + L4 * L5) * A)) * sABi3;
    double gz = (dCz * AB - C * ((r21.x * M6 - r21.y * M3) * B + (M1 * M2 + M4 * M5) * A)) * sABi3;
    double den = sqrt(1.0 - W * W);
    double f = (den == 0.0) ? 1.0 / 1E-10 : 1.0 / den;
    return scl(d3(f * gx, f * gy, f * gz), -1.0);
}

// (int) of a float with x86-64 semantics (NaN / out of range -> INT_MIN), so an invalid table
// index is rejected the way the reference's x86-64 build rejects it.
__device__ __forceinline__ int f2i_x86(float x) {
    if(!(x > -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int)x;
}

// calcIndexOfLowerPointOfInterpolationLine (FunctorCalcForce.cpp:426-430)
__device__ __forceinline__ int tindex(float x, const float* tab) {
    float delta = (tab[3 * (kNpts - 1)] - tab[0]) / float(kNpts - 1);
    return f2i_x86((x - tab[0]) / delta);
}

// interpolateLinear (FunctorCalcForce.cpp:457-465)
__device__ __forceinline__ float interp(float r, float x1, float y1, float x2, float y2) {
    float denom = x1 - x2;
    if(denom == 0.0f) denom = 3.0f * FLT_MIN;
    float a = (y1 - y2) / denom;
    float b = y1 - a * x1;
    return (a * r + b);
}

__device__ float calc_angle(D3 rk, D3 ri, D3 rj) {
    D3 rik = sub(rk, ri), rij = sub(rj, ri);
    float dp = (float)dotp(rik, rij);
    float RR = (float)nrm(rik) * (float)nrm(rij);
    float c = (RR != 0.0f) ? dp / RR : 1.0f;
    return (float)acos((double)c);
}

__device__ float calc_dihedral(D3 rk, D3 ri, D3 rj, D3 rl) {
    D3 rik = sub(rk, ri), rij = sub(rj, ri), rjl = sub(rl, rj);
    D3 n1 = crs(rik, rij), n2 = crs(rij, rjl);
    float dp = (float)dotp(n1, n2);
    float nn = (float)nrm(n1) * (float)nrm(n2);
    float c = (nn != 0.0f) ? dp / nn : 1.0f;
    if(c < -1.0f) c = -1.0f;
    if(c > 1.0f) c = 1.0f;
    return (float)acos((double)c);
}

// scaleForcesAndPotentials (FunctorCalcForce.cpp:95-157) as a (applies, factor) pair.
__device__ __forceinline__ bool exclusion(const DevSys& d, const Params& P, int k, int i, float& f) {
    for(int e = d.bptr[k]; e < d.bptr[k + 1]; e++) if(d.bj[e] == i) { f = P.scale12; return true; }
    for(int e = d.aptr[k]; e < d.aptr[k + 1]; e++) if(!d.acen[e] && d.aj[e] == i) { f = P.scale13; return true; }
    for(int e = d.dptr[k]; e < d.dptr[k + 1]; e++) if(!d.dcen[e] && d.dl[e] == i) { f = P.scale14; return true; }
    const int mi = d.mol[i], mk = d.mol[k];
    if(mi >= 0 && mk >= 0 && mi == mk) { f = P.scale1N; return true; }
    return false;
}

// ---------------------------------------------------------------------------------------------
// Cell list (CFunctorGenCellList::operator() and kernelAssembleList)
// ---------------------------------------------------------------------------------------------
__global__ void k_cell_assign(DevSys d, Params P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n) return;
    const float wx = box_f(d, P, 0), wy = box_f(d, P, 1), wz = box_f(d, P, 2);
    const float lx = -wx / 2.0f, ly = -wy / 2.0f, lz = -wz / 2.0f;
    const int Nx = P.nx, Ny = P.ny, Nz = P.nz;
    int ix = (int)floor((d.r[3 * i] - double(lx)) * double(Nx) / double(wx));
    int iy = (int)floor((d.r[3 * i + 1] - double(ly)) * double(Ny) / double(wy));
    int iz = (int)floor((d.r[3 * i + 2] - double(lz)) * double(Nz) / double(wz));
    ix = (ix < 0) ? 0 : ((ix >= Nx) ? Nx - 1 : ix);
    iy = (iy < 0) ? 0 : ((iy >= Ny) ? Ny - 1 : iy);
    iz = (iz < 0) ? 0 : ((iz >= Nz) ? Nz - 1 : iz);
    d.atom_cell[3 * i] = ix;
    d.atom_cell[3 * i + 1] = iy;
    d.atom_cell[3 * i + 2] = iz;
    atomicAdd(&d.cell_count[ix + Nx * (iy + iz * Ny)], 1);
    // FP32 copy of the positions for the neighbour-list prefilter (absent in the context-free
    // neighbour list, which then decides every candidate in FP64)
    if(d.rb4) d.rb4[i] = make_float4((float)d.r[3 * i], (float)d.r[3 * i + 1], (float)d.r[3 * i + 2], 0.0f);
}

// Exclusive scan of the cell counts in one block; empty cells get first = -1 (CListPointer default).
__global__ void k_cell_scan(DevSys d, int ncell) {
    __shared__ int warp_tot[32];
    __shared__ int carry;
    if(threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for(int base = 0; base < ncell; base += blockDim.x) {
        const int c = base + threadIdx.x;
        const int v = (c < ncell) ? d.cell_count[c] : 0;
        int x = v;
        for(int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if(lane >= o) x += y;
        }
        if(lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if(warp == 0) {
            int t = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0;
            for(int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, t, o);
                if(lane >= o) t += y;
            }
            warp_tot[lane] = t;
        }
        __syncthreads();
        const int excl = carry + (warp ? warp_tot[warp - 1] : 0) + x - v;
        if(c < ncell) {
            d.cell_first[c] = (v != 0) ? excl : -1;
            d.cell_cursor[c] = 0;
        }
        __syncthreads();
        if(threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
}

__global__ void k_cell_scatter(DevSys d, Params P, int* tmp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n) return;
    const int c = d.atom_cell[3 * i] + P.nx * (d.atom_cell[3 * i + 1] + d.atom_cell[3 * i + 2] * P.ny);
    const int slot = atomicAdd(&d.cell_cursor[c], 1);
    tmp[d.cell_first[c] + slot] = i;
}

// One warp per cell: place each atom at its rank (number of smaller indices in the cell), which
// is the reference's serial order (ascending atom index within a cell).
__global__ void k_cell_rank(DevSys d, int ncell, const int* tmp) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if(warp >= ncell) return;
    const int cnt = d.cell_count[warp], first = d.cell_first[warp];
    for(int a = lane; a < cnt; a += 32) {
        const int v = tmp[first + a];
        int rank = 0;
        for(int b = 0; b < cnt; b++) rank += (tmp[first + b] < v);
        d.cell_list[first + rank] = v;
    }
}

// ---------------------------------------------------------------------------------------------
// Full neighbour list in the reference order (CFunctorGenNeighList::operator()), one warp per
// atom: the 27 cells in the reference's loop order, each cell's atoms 32 at a time, accepted ones
// compacted in order with a ballot.  The distance test is first made in FP32 from the FP32 copy
// of the positions; only a candidate whose FP32 squared distance lies within 0.4 % of rc^2 (the
// FP32 error is below 0.01 % for boxes up to a few hundred A) is decided by the reference's FP64
// arithmetic, so the accepted set is exactly the reference's.
// ---------------------------------------------------------------------------------------------
// The reference's FP64 distance test of one candidate (FunctorGenNeighList.cpp:72-151), out of
// line: warps reach it only for candidates within 0.4 % of rc^2 in FP32.
__device__ __noinline__ bool neigh_test_fp64(double x0, double y0, double z0, const double* rj, const double* w,
                                             double rc2) {
    double dX = x0 - rj[0], dY = y0 - rj[1], dZ = z0 - rj[2];
    dX = (dX < 0.0) ? -dX : dX;
    dY = (dY < 0.0) ? -dY : dY;
    dZ = (dZ < 0.0) ? -dZ : dZ;
    if(dX > (w[0] / 2.0)) dX = w[0] - dX;
    if(dY > (w[1] / 2.0)) dY = w[1] - dY;
    if(dZ > (w[2] / 2.0)) dZ = w[2] - dZ;
    return (dX * dX + dY * dY + dZ * dZ) < rc2;
}

// Constants of the list kernel, computed once per block into shared memory (in registers the
// compiler recomputed them with FP64 conversions inside the candidate loop).
struct NeighConst {
    double w[3];
    double rc2;
    float wf[3], hf[3];
    float lo2, hi2;
};

__global__ void k_neigh(DevSys d, Params P, float rc) {
    __shared__ NeighConst nc;
    if(threadIdx.x == 0) {
        float rc2f = rc;
        rc2f *= rc2f;
        nc.rc2 = (double)rc2f;
        const float Bx = box_f(d, P, 0), By = box_f(d, P, 1), Bz = box_f(d, P, 2);
        const float lx = -Bx / 2.0f, ly = -By / 2.0f, lz = -Bz / 2.0f;
        nc.w[0] = double(lx + Bx) - double(lx);
        nc.w[1] = double(ly + By) - double(ly);
        nc.w[2] = double(lz + Bz) - double(lz);
        for(int a = 0; a < 3; a++) {
            nc.wf[a] = (float)nc.w[a];
            nc.hf[a] = 0.5f * nc.wf[a];
        }
        nc.lo2 = (float)(nc.rc2 * 0.996);
        nc.hi2 = (float)(nc.rc2 * 1.004);
    }
    __syncthreads();
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if(k >= P.n) return;
    const float lo2 = nc.lo2, hi2 = nc.hi2;
    const int Nx = P.nx, Ny = P.ny, Nz = P.nz;
    const double x0 = d.r[3 * k], y0 = d.r[3 * k + 1], z0 = d.r[3 * k + 2];
    const bool pre = d.rb4 != nullptr;
    const float4 rk = pre ? d.rb4[k] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int cx = d.atom_cell[3 * k], cy = d.atom_cell[3 * k + 1], cz = d.atom_cell[3 * k + 2];
    int c = 0;
    int* out = d.nbr_list + (size_t)k * d.nbr_max;
    // the entries whose type pair has a non-bonded term, in list order, for the force gather (the
    // others add exactly zero there)
    const bool keep_nb = d.nbr_list_nb != nullptr;
    int c_nb = 0;
    int* out_nb = keep_nb ? d.nbr_list_nb + (size_t)k * d.nbr_max : nullptr;
    const int* cnt_row = keep_nb ? d.nb_cnt + d.type[k] * P.T : nullptr;
    for(int ix = cx - 1; ix <= cx + 1; ix++) {
        const int Ix = (ix >= 0) ? ((ix < Nx) ? ix : 0) : Nx - 1;
        for(int iy = cy - 1; iy <= cy + 1; iy++) {
            const int Iy = (iy >= 0) ? ((iy < Ny) ? iy : 0) : Ny - 1;
            for(int iz = cz - 1; iz <= cz + 1; iz++) {
                const int Iz = (iz >= 0) ? ((iz < Nz) ? iz : 0) : Nz - 1;
                const int cell = Ix + Nx * (Iy + Iz * Ny);
                const int cnt = d.cell_count[cell], first = d.cell_first[cell];
                for(int base = 0; base < cnt; base += 32) {
                    bool take = false;
                    int j = 0;
                    if(base + lane < cnt) {
                        j = d.cell_list[first + base + lane];
                        float f2 = 0.5f * (lo2 + hi2);   // without the FP32 copy: always the FP64 test
                        if(pre) {
                            const float4 rj = d.rb4[j];
                            float fX = fabsf(rk.x - rj.x), fY = fabsf(rk.y - rj.y), fZ = fabsf(rk.z - rj.z);
                            if(fX > nc.hf[0]) fX = nc.wf[0] - fX;
                            if(fY > nc.hf[1]) fY = nc.wf[1] - fY;
                            if(fZ > nc.hf[2]) fZ = nc.wf[2] - fZ;
                            f2 = fX * fX + fY * fY + fZ * fZ;
                        }
                        if(f2 < lo2) {
                            take = true;
                        } else if(f2 <= hi2) {
                            take = neigh_test_fp64(x0, y0, z0, d.r + 3 * j, nc.w, nc.rc2);
                        }
                        take = take && (j != k);
                    }
                    const unsigned ball = __ballot_sync(0xffffffffu, take);
                    if(take) {
                        const int slot = c + __popc(ball & ((1u << lane) - 1u));
                        if(slot < d.nbr_max) out[slot] = j;
                    }
                    c += __popc(ball);
                    if(keep_nb) {
                        const bool nb = take && cnt_row[d.type[j]] > 0;
                        const unsigned bnb = __ballot_sync(0xffffffffu, nb);
                        if(nb) {
                            const int slot = c_nb + __popc(bnb & ((1u << lane) - 1u));
                            if(slot < d.nbr_max) out_nb[slot] = j;
                        }
                        c_nb += __popc(bnb);
                    }
                }
            }
        }
    }
    if(lane == 0) {
        d.nbr_count[k] = c;
        if(keep_nb) d.nbr_count_nb[k] = c_nb;
        if(c > d.nbr_max) {
            d.sc->overflow = 1;
            atomicMax(&d.sc->needed, c);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Per-atom force/energy gather, table mode (CFunctorCalcForce::operator())
// ---------------------------------------------------------------------------------------------
// ---------------------------------------------------------------------------------------------
// Exact FP64 results with little FP64 work, for the all-pairs Coulomb loop.  On this GPU an FP64
// instruction occupies the FP64 pipe for a whole warp, and that pipe bounds the loop.  The pair's
// float distance R and its FP64 quotient K / R^3 are therefore reached with FP32 and integer
// instructions, bit-identical to the reference's FP64 arithmetic: each result is decided with a
// margin far above the error of its FP32 evaluation, and the rare operands too close to a
// rounding boundary (or outside the ranges the argument covers) take the FP64 operations.
// ---------------------------------------------------------------------------------------------

// The FP64 operations themselves.  Not inlined: a call is a branch that warps skip when no lane
// needs it, where inlined code could be predicated and would then occupy the FP64 pipe on every
// pass.
__device__ __noinline__ float dist_fp64(double x, double y, double z) { return (float)sqrt(x * x + y * y + z * z); }
__device__ __noinline__ double quot_fp64(float K, float R) { return (double)K / (double)R; }

// x = hi + lo with hi the float of x's leading 24 bits (exact) and lo the float of the remaining
// 29 (rounded); false when x is neither zero nor in [2^-60, 2^60].
__device__ __forceinline__ bool split_df(double x, float& hi, float& lo) {
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if((b & 0x7fffffffffffffffLL) == 0) {
        hi = lo = 0.0f;
        return true;
    }
    if(ex < 1023 - 60 || ex > 1023 + 60) return false;
    const uint32_t sgn = (uint32_t)((unsigned long long)b >> 63) << 31;
    hi = __uint_as_float(sgn | ((uint32_t)(ex - 1023 + 127) << 23) | (uint32_t)((b >> 29) & 0x7fffff));
    const float l = __fmul_rn(__uint2float_rn((uint32_t)(b & 0x1fffffff)), __uint_as_float((uint32_t)(ex - 1075 + 127) << 23));
    lo = __uint_as_float(__float_as_uint(l) | sgn);
    return true;
}

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& t) {
    const float ss = __fadd_rn(a, b), bb = __fsub_rn(ss, a);
    s = ss;
    t = __fadd_rn(__fsub_rn(a, __fsub_rn(ss, bb)), __fsub_rn(b, bb));
}

// R = (float)sqrt(x*x + y*y + z*z) as the reference evaluates it in FP64 (its norm, then the
// conversion), bit for bit.  S = x^2 + y^2 + z^2 is formed as a float pair Sh + Sl from the
// components' hi/lo splits (hi^2 exactly by fma, the cross and lo terms in FP32) to about 2^-44
// relative, which covers the reference's own FP64 roundings of S (about 2^-52).  For the candidate
// a = RN(sqrt(Sh)) the residual S - a^2 = fma(-a, a, Sh) + Sl places sqrt(S) against a's rounding
// interval (a - D/2, a + U/2), D and U the float spacings below and above a: in residual terms
// -(a D - D^2/4) < S - a^2 < a U + U^2/4.  A residual inside by a relative margin of 2^-12 decides
// R = a; one step to a neighbouring float is decided the same way; the rest (including any S
// within 2^-52 of a midpoint square, where the FP64 rounding of the root could land on the
// midpoint) takes the FP64 evaluation.
__device__ __forceinline__ float dist_to_float(double x, double y, double z) {
    float xh, xl, yh, yl, zh, zl;
    if(!split_df(x, xh, xl) || !split_df(y, yh, yl) || !split_df(z, zh, zl)) return dist_fp64(x, y, z);
    const float px = __fmul_rn(xh, xh), ex = __fmaf_rn(xh, xh, -px);
    const float py = __fmul_rn(yh, yh), ey = __fmaf_rn(yh, yh, -py);
    const float pz = __fmul_rn(zh, zh), ez = __fmaf_rn(zh, zh, -pz);
    float s1, t1, s2, t2;
    two_sum_f(px, py, s1, t1);
    two_sum_f(s1, pz, s2, t2);
    const float cross = __fadd_rn(__fadd_rn(__fmul_rn(xh, xl), __fmul_rn(yh, yl)), __fmul_rn(zh, zl));
    const float low = __fadd_rn(__fadd_rn(__fmul_rn(xl, xl), __fmul_rn(yl, yl)), __fmul_rn(zl, zl));
    const float c = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(t1, t2), __fadd_rn(__fadd_rn(ex, ey), ez)),
                                        __fmul_rn(2.0f, cross)), low);
    const float Sh = __fadd_rn(s2, c), Sl = __fsub_rn(c, __fsub_rn(Sh, s2));
    if(!(Sh >= 0x1p-100f)) {
        // all three components +-0 (compared as bit patterns, without FP64 instructions): R = 0
        if(((__double_as_longlong(x) | __double_as_longlong(y) | __double_as_longlong(z)) & 0x7fffffffffffffffLL) == 0)
            return 0.0f;
        return dist_fp64(x, y, z);
    }
    const float lo = 1.0f - 0x1p-12f, hi = 1.0f + 0x1p-12f;
    const float a = __fsqrt_rn(Sh);
    const float Er = __fadd_rn(__fmaf_rn(-a, a, Sh), Sl);
    const uint32_t ab = __float_as_uint(a);
    const float U = __uint_as_float((ab & 0x7f800000u) - (23u << 23));
    const float D = ((ab & 0x7fffffu) == 0) ? 0.5f * U : U;
    const float tu = __fmul_rn(a, U), td = __fmul_rn(a, D);
    if(Er < tu * lo && Er > -td * lo) return a;
    if(Er > tu * hi || Er < -td * hi) {
        const bool up = Er > 0.0f;
        const float a1 = __uint_as_float(up ? ab + 1u : ab - 1u);
        const uint32_t b1 = __float_as_uint(a1);
        const float U1 = __uint_as_float((b1 & 0x7f800000u) - (23u << 23));
        const float D1 = ((b1 & 0x7fffffu) == 0) ? 0.5f * U1 : U1;
        const float Er1 = up ? __fsub_rn(Er, 2.0f * tu) : __fadd_rn(Er, 2.0f * td);   // S - a1^2, up to U^2 or D^2
        if(Er1 < __fmul_rn(a1, U1) * lo && Er1 > -__fmul_rn(a1, D1) * lo) return a1;
    }
    return dist_fp64(x, y, z);
}

// (double)K / (double)R3 for floats, the correctly rounded FP64 quotient, bit for bit.  On |K|:
// q1 = RN(K / R3) and q2 = RN(r1 / R3) are correctly rounded FP32 quotients, so the remainders
// r1 = K - R3 q1 and r2 = r1 - R3 q2 are exact as fused multiply-adds (with the operand ranges
// below none of them underflows), and q3 = r2 (1 / R3) has relative error <= 2^-23.  The sum
// q1 + q2 + q3 is assembled in a 128-bit integer with 72 bits below q1's last bit, where the
// truncations and q3's error stay below 8 units; rounded to 53 bits it is the FP64 quotient unless
// its rounding bits lie within 16 units of the half-way point, which then takes the FP64 division.
// (A quotient of two floats is never an FP64 midpoint, so no tie arises.)
__device__ __forceinline__ double quot_ff(float K, float R) {
    const uint32_t kb = __float_as_uint(K), rb = __float_as_uint(R);
    const int ke = (int)((kb >> 23) & 0xff), re = (int)((rb >> 23) & 0xff);
    if(ke < 127 - 60 || ke > 127 + 60 || re < 127 - 60 || re > 127 + 60 || ke - re < -40 || ke - re > 40 || (rb >> 31))
        return quot_fp64(K, R);
    const float Ka = __uint_as_float(kb & 0x7fffffffu);
    const float q1 = __fdiv_rn(Ka, R);
    const float r1 = __fmaf_rn(-R, q1, Ka);
    const float q2 = __fdiv_rn(r1, R);
    const float r2 = __fmaf_rn(-R, q2, r1);
    const float q3 = __fmul_rn(r2, __frcp_rn(R));
    const uint32_t b1 = __float_as_uint(q1);
    const int e1 = (int)(b1 >> 23);
    unsigned __int128 V = (unsigned __int128)((b1 & 0x7fffffu) | 0x800000u) << 72;
#pragma unroll
    for(int i = 0; i < 2; i++) {
        const uint32_t bf = __float_as_uint(i == 0 ? q2 : q3);
        if((bf & 0x7fffffffu) == 0) continue;
        const int ef = (int)((bf >> 23) & 0xff);
        const unsigned __int128 M = (unsigned __int128)((bf & 0x7fffffu) | 0x800000u);
        const int sh = ef - e1 + 72;
        const unsigned __int128 c = sh >= 0 ? (M << sh) : (sh > -64 ? (M >> (-sh)) : (unsigned __int128)0);
        if(bf >> 31) V -= c;
        else V += c;
    }
    if(!(V >> 94)) return quot_fp64(K, R);
    const int msb = (V >> 95) ? 95 : 94;
    const int drop = msb - 52;
    unsigned long long sig = (unsigned long long)(V >> drop);
    const unsigned __int128 rem = V & (((unsigned __int128)1 << drop) - 1);
    const unsigned __int128 half = (unsigned __int128)1 << (drop - 1);
    if(rem + 16 >= half && rem <= half + 16) return quot_fp64(K, R);
    if(rem > half) sig++;
    const unsigned long long bits = ((unsigned long long)(msb + e1 - 222 + 1023) << 52) + sig - (1ULL << 52);
    return __longlong_as_double((long long)(bits | ((unsigned long long)(kb >> 31) << 63)));
}

// Box widths of the minimum image: w, -w, w/2 (bits, and rounded to float) per axis.  Kept in
// shared memory by the Coulomb kernel, so that the loop reads them instead of recomputing them
// with FP64 operations when registers run short.
struct BoxImage {
    double w[3], nw[3];
    long long hw[3];
    float hwf[3];
};

// x truncated to a float (relative error < 2^-23; |x| < 2^-126 gives 0, larger than the float
// range or NaN gives NaN, on which every comparison below is false).
__device__ __forceinline__ float trunc_f(double x) {
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    const uint32_t sgn = (uint32_t)((unsigned long long)b >> 63) << 31;
    if(ex <= 0) return __uint_as_float(sgn);
    if(ex >= 255) return __uint_as_float(sgn | 0x7fc00000u);
    return __uint_as_float(sgn | ((uint32_t)ex << 23) | (uint32_t)((b >> 29) & 0x7fffff));
}

// The image shift of moveToSameSideOfPBCAsThis from the FP64 test itself: |c - v| > w/2 compared
// as bit patterns, the direction from the sign of c - v.
__device__ __noinline__ double image_shift_fp64(double c, double v, const BoxImage& bx, int a) {
    const long long db = __double_as_longlong(c - v);
    if((db & 0x7fffffffffffffffLL) > bx.hw[a]) return (db >= 0) ? bx.w[a] : bx.nw[a];
    return -0.0;
}

// One axis of moveToSameSideOfPBCAsThis (Utilities/3DVector.cpp:133-165) followed by the
// separation c - v.  The test |c - v| > w/2 runs on the float truncations cf, vf: their
// difference is within 1.5 2^-23 (|cf| + |vf|) of c - v, so a margin of 2^-20 (|cf| + |vf| + w/2)
// decides it, and only separations within the margin of w/2 take the FP64 test.  The shift is
// then one FP64 addition for every lane: v + (-0.0) is v for every v, signed zeros included.
__device__ __forceinline__ double image_sep(double c, double v, float cf, float vf, const BoxImage& bx, int a) {
    const float d = fabsf(__fsub_rn(cf, vf));
    const float m = __fmul_rn(0x1p-20f, __fadd_rn(__fadd_rn(fabsf(cf), fabsf(vf)), bx.hwf[a]));
    double ws;
    if(d > __fadd_rn(bx.hwf[a], m)) ws = (cf > vf) ? bx.w[a] : bx.nw[a];
    else if(d < __fsub_rn(bx.hwf[a], m)) ws = -0.0;
    else ws = image_shift_fp64(c, v, bx, a);
    return c - (v + ws);
}

// The exclusion scaling of a pair's force (rare: bonded partners and same-molecule pairs), out of
// line for the same reason as the FP64 fallbacks above.
__device__ __noinline__ D3 scale_fp64(D3 f, float sc) { return scl(f, (double)sc); }

// Coulomb term of the pair (k, i) (FunctorCalcForce.cpp:258-278, 514-535) in the reference's
// arithmetic: float R from the FP64 minimum-image separation, FP64 K / R^3, the pair energy on
// the lower index, the exclusion scaling.
__device__ __forceinline__ void coulomb_pair(const DevSys& d, const Params& P, int k, int i, const D3& rk, D3 ri,
                                             const float* rkf, const float* rif, float qk, float qi, int molk,
                                             int moli, bool local, const BoxImage& bx, D3& f, float& u) {
    u = 0.0f;
    const D3 rv = d3(image_sep(rk.x, ri.x, rkf[0], rif[0], bx, 0), image_sep(rk.y, ri.y, rkf[1], rif[1], bx, 1),
                     image_sep(rk.z, ri.z, rkf[2], rif[2], bx, 2));
    const float R = dist_to_float(rv.x, rv.y, rv.z);
    const float R3 = R * R * R;
    const float K = kCoulombKf * qk * qi;
    if((i > k) && (R != 0.0f)) u += K / R;
    f = (R3 != 0.0f) ? scl(rv, quot_ff(K, R3)) : d3(0, 0, 0);
    // pairs of different molecules have no exclusion when none of k's partners lies outside its
    // molecule; otherwise the reference's search
    float sc;
    if(!(local && moli != molk) && exclusion(d, P, k, i, sc)) {
        f = scale_fp64(f, sc);
        u *= sc;
    }
}

constexpr int kRefTile = 64;    // threads per block of the bonded gather (spread over every SM)
constexpr int kSrJ = 16;         // list positions per tile of the short-range kernel
constexpr int kSrW = 16;         // its pair warps (kSrJ / kSrW positions each per tile)

// Bonded terms, one thread per atom (atoms taken by type), each sum in the reference's order
// (bonds, angles, dihedrals).  The sums are stored in F and U; the short-range and the all-pairs
// Coulomb kernels continue them.
__global__ void __launch_bounds__(kRefTile) k_force(DevSys d, Params P) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = (d.force_order && tid < P.n) ? d.force_order[tid] : tid;
    const float Lf[3] = {box_f(d, P, 0), box_f(d, P, 1), box_f(d, P, 2)};
    const double w[3] = {double(Lf[0]) / 2.0 - (-double(Lf[0]) / 2.0), double(Lf[1]) / 2.0 - (-double(Lf[1]) / 2.0),
                         double(Lf[2]) / 2.0 - (-double(Lf[2]) / 2.0)};
    if(d.sc->overflow) return;   // neighbour list incomplete: the step is redone after growing it
    const bool act = k < P.n;
    const bool live = act && d.mobile[k];
    double Fx = 0.0, Fy = 0.0, Fz = 0.0;
    float Uk = 0.0f;
    const D3 rk = live ? load3(d.r, k) : d3(0, 0, 0);
    if(live) {
        // bonds
        for(int e = d.bptr[k]; e < d.bptr[k + 1]; e++) {
            const int i = d.bj[e];
            D3 ri = load3(d.r, i);
            same_side(rk, ri, w);
            const float* tab = d.bond_tab + (size_t)d.bt[e] * kNpts * 3;
            const float rr = (float)nrm(sub(rk, ri));
            const int idx = tindex(rr, tab);
            float md = 0.0f;
            if(idx >= 0 && idx < kNpts - 1) {
                const float* p1 = tab + 3 * idx;
                const float* p2 = p1 + 3;
                md += interp(rr, p1[0], p1[1], p2[0], p2[1]);
                if(i > k) Uk += interp(rr, p1[0], p1[2], p2[0], p2[2]);
            }
            const D3 f = scl(coeff12(ri, rk), (double)md);
            Fx += f.x; Fy += f.y; Fz += f.z;
        }
        // angles
        for(int e = d.aptr[k]; e < d.aptr[k + 1]; e++) {
            D3 ri = load3(d.r, d.ai[e]), rj = load3(d.r, d.aj[e]);
            same_side(rk, ri, w);
            same_side(rk, rj, w);
            const float* tab = d.angle_tab + (size_t)d.at[e] * kNpts * 3;
            D3 f;
            if(d.acen[e]) {
                const float th = calc_angle(ri, rk, rj);
                const int idx = tindex(th, tab);
                float md = 0.0f;
                if(idx >= 0 && idx < kNpts - 1) {
                    const float* p1 = tab + 3 * idx;
                    const float* p2 = p1 + 3;
                    md += interp(th, p1[0], p1[1], p2[0], p2[1]);
                    Uk += interp(th, p1[0], p1[2], p2[0], p2[2]);
                }
                f = scl(coeff_ang2(rj, rk, ri), (double)md);
            } else {
                const float th = calc_angle(rk, ri, rj);
                const int idx = tindex(th, tab);
                float md = 0.0f;
                if(idx >= 0 && idx < kNpts - 1) {
                    const float* p1 = tab + 3 * idx;
                    const float* p2 = p1 + 3;
                    md += interp(th, p1[0], p1[1], p2[0], p2[1]);
                }
                f = scl(coeff_ang13(rj, ri, rk), (double)md);
            }
            Fx += f.x; Fy += f.y; Fz += f.z;
        }
        // dihedrals
        for(int e = d.dptr[k]; e < d.dptr[k + 1]; e++) {
            D3 ri = load3(d.r, d.di[e]), rj = load3(d.r, d.dj[e]), rl = load3(d.r, d.dl[e]);
            same_side(rk, ri, w);
            same_side(rk, rj, w);
            same_side(rk, rl, w);
            const float* tab = d.dih_tab + (size_t)d.dt[e] * kNpts * 3;
            D3 f;
            if(d.dcen[e]) {
                const float th = calc_dihedral(ri, rk, rj, rl);
                const int idx = tindex(th, tab);
                float md = 0.0f;
                if(idx >= 0 && idx < kNpts - 1) {
                    const float* p1 = tab + 3 * idx;
                    const float* p2 = p1 + 3;
                    md += interp(th, p1[0], p1[1], p2[0], p2[1]);
                    Uk += 0.5f * interp(th, p1[0], p1[2], p2[0], p2[2]);
                }
                f = scl(coeff_dih23(rl, rj, rk, ri), (double)md);
            } else {
                const float th = calc_dihedral(rk, ri, rj, rl);
                const int idx = tindex(th, tab);
                float md = 0.0f;
                if(idx >= 0 && idx < kNpts - 1) {
                    const float* p1 = tab + 3 * idx;
                    const float* p2 = p1 + 3;
                    md += interp(th, p1[0], p1[1], p2[0], p2[1]);
                }
                f = scl(coeff_dih14(rl, rj, ri, rk), (double)md);
            }
            Fx += f.x; Fy += f.y; Fz += f.z;
        }
    }
    if(!act) return;
    d.F[3 * k] = Fx;
    d.F[3 * k + 1] = Fy;
    d.F[3 * k + 2] = Fz;
    d.U[k] = live ? (double)Uk : 0.0;
}

// Short-range term of the list entry (k, i) in the reference's arithmetic (FunctorCalcForce.cpp:
// 159-256): the FP64 minimum-image separation r12 = rk - ri, the float distance of its FP64
// norm, the tabulated terms of the pair's type, the force coeff12 (r12 / |r12|, FP64) times their
// sum, the pair energy on the lower index, the exclusion scaling.
__device__ __forceinline__ void sr_pair(const DevSys& d, const Params& P, int k, int i, const D3& rk, const float* rkf,
                                        int pair_row, bool local_k, int molk, const BoxImage& bx, D3& f, float& u) {
    u = 0.0f;
    const D3 ri = load3(d.r, i);
    const float rif[3] = {trunc_f(ri.x), trunc_f(ri.y), trunc_f(ri.z)};
    const D3 rv = d3(image_sep(rk.x, ri.x, rkf[0], rif[0], bx, 0), image_sep(rk.y, ri.y, rkf[1], rif[1], bx, 1),
                     image_sep(rk.z, ri.z, rkf[2], rif[2], bx, 2));
    const double R = sqrt(rv.x * rv.x + rv.y * rv.y + rv.z * rv.z);
    const float rr = (float)R;
    f = d3(0, 0, 0);
    if(!(rr < 1E-3f)) {
        float sum = 0.0f;
        const int pair = pair_row + d.type[i];
        const int cnt = d.nb_cnt[pair];
        for(int ff = 0; ff < cnt; ff++) {
            const float* tab = d.nb_tab + ((size_t)pair * kMaxFF + ff) * kNpts * 3;
            const int idx = tindex(rr, tab);
            if(idx >= 0 && idx < kNpts - 1) {
                const float* p1 = tab + 3 * idx;
                const float* p2 = p1 + 3;
                sum += interp(rr, p1[0], p1[1], p2[0], p2[1]);
                if(i > k) u += interp(rr, p1[0], p1[2], p2[0], p2[2]);
            }
        }
        f = scl(scl(rv, 1.0 / R), (double)sum);
    }
    float sc;
    if(!(local_k && d.mol[i] != molk) && exclusion(d, P, k, i, sc)) {
        f = scale_fp64(f, sc);
        u *= sc;
    }
}

// Short-range terms from the neighbour list (FunctorCalcForce.cpp:234-256), continuing each atom's
// sums after its bonded terms, in list order.  Only the entries whose type pair has a non-bonded
// term are visited: the others add the force coeff12 * 0.0 = +-0 and no energy, which leaves a sum
// that starts at +0 unchanged.  Layout as the all-pairs Coulomb kernel below: a block owns 32
// atoms (taken by type, so that the lanes meet the same terms); its first kCoulW warps compute
// the terms of list positions e (lane = atom) and park them in shared memory, and the last warp
// adds each tile's terms in ascending e one tile behind.
__global__ void __launch_bounds__(32 * (kSrW + 1)) k_sr_parked(DevSys d, Params P) {
    __shared__ double tfx[2][kSrJ][32], tfy[2][kSrJ][32], tfz[2][kSrJ][32];
    __shared__ float tu[2][kSrJ][32];
    __shared__ unsigned ton[2][kSrJ];
    __shared__ BoxImage bx;
    if(d.sc->overflow) return;   // the step is redone after the neighbour list grows
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = P.n;
    const int slot = blockIdx.x * 32 + lane;
    const int k = slot < n ? (d.force_order ? d.force_order[slot] : slot) : n;
    const bool live = k < n && d.mobile[k];
    const bool nb_only = d.nbr_list_nb != nullptr;
    const int cnt = live ? min(nb_only ? d.nbr_count_nb[k] : d.nbr_count[k], d.nbr_max) : 0;
    const int mx = __reduce_max_sync(0xffffffffu, cnt);
    if(!__syncthreads_or(mx > 0)) return;
    if(threadIdx.x < 3) {
        const int a = threadIdx.x;
        const float Lf = box_f(d, P, a);
        const double w = double(Lf) / 2.0 - (-double(Lf) / 2.0);
        bx.w[a] = w;
        bx.nw[a] = -w;
        bx.hw[a] = __double_as_longlong(w / 2.0);
        bx.hwf[a] = __double2float_rn(w / 2.0);
    }
    const int ntile = (mx + kSrJ - 1) / kSrJ;
    if(warp < kSrW) {
        const D3 rk = cnt > 0 ? load3(d.r, k) : d3(0, 0, 0);
        const float rkf[3] = {trunc_f(rk.x), trunc_f(rk.y), trunc_f(rk.z)};
        const int* nl = (nb_only ? d.nbr_list_nb : d.nbr_list) + (size_t)(k < n ? k : 0) * d.nbr_max;
        const int pair_row = cnt > 0 ? d.type[k] * P.T : 0;
        const bool local_k = cnt > 0 && d.excl_local[k] != 0;
        const int molk = cnt > 0 ? d.mol[k] : -1;
        __syncthreads();
        for(int t = 0; t < ntile; t++) {
            const int b = t & 1;
#pragma unroll
            for(int h = 0; h < kSrJ / kSrW; h++) {
                const int jj = warp + h * kSrW;
                const int e = t * kSrJ + jj;
                const bool on = e < cnt;
                D3 f = d3(0, 0, 0);
                float u = 0.0f;
                if(on) sr_pair(d, P, k, nl[e], rk, rkf, pair_row, local_k, molk, bx, f, u);
                const unsigned m = __ballot_sync(0xffffffffu, on);
                if(on) {
                    tfx[b][jj][lane] = f.x;
                    tfy[b][jj][lane] = f.y;
                    tfz[b][jj][lane] = f.z;
                    tu[b][jj][lane] = u;
                }
                if(lane == 0) ton[b][jj] = m;
            }
            __syncthreads();
        }
        __syncthreads();   // the summing warp's last tile
    } else {
        double Fx = 0.0, Fy = 0.0, Fz = 0.0;
        float Uk = 0.0f;
        if(cnt > 0) {
            Fx = d.F[3 * k];
            Fy = d.F[3 * k + 1];
            Fz = d.F[3 * k + 2];
            Uk = (float)d.U[k];   // stored as double from a float: exact
        }
        __syncthreads();
        for(int t = 0; t <= ntile; t++) {
            if(t > 0) {
                const int b = (t - 1) & 1;
                for(int jj = 0; jj < kSrJ; jj++) {
                    if((ton[b][jj] >> lane) & 1u) {
                        Fx += tfx[b][jj][lane];
                        Fy += tfy[b][jj][lane];
                        Fz += tfz[b][jj][lane];
                        Uk += tu[b][jj][lane];
                    }
                }
            }
            __syncthreads();
        }
        if(cnt > 0) {
            d.F[3 * k] = Fx;
            d.F[3 * k + 1] = Fy;
            d.F[3 * k + 2] = Fz;
            d.U[k] = (double)Uk;
        }
    }
}

// All-pairs Coulomb, minimum image, no cutoff (FunctorCalcForce.cpp:258-278, 514-535), continuing
// each atom's sums after its bonded and short-range terms.
//
// A block owns 32 atoms.  Its first kCoulW warps compute the pair terms of those atoms (lane =
// atom) against a tile of kCoulJ positions, two positions per warp, and park them in shared
// memory; the last warp adds the parked terms of the previous tile to the atoms' sums in
// ascending j.  Every sum therefore keeps the reference's order i = 0 .. N-1 while the FP64 pair
// arithmetic, the cost of this kernel (on this GPU an FP64 instruction occupies its pipe for the
// whole warp), is spread over nine warps per 32 atoms and over every SM.  A pair whose charge
// product K is zero adds exactly +-0 to every sum and is skipped (all pairs of an atom whose own
// charge is zero), as the reference's arithmetic leaves those sums unchanged.
constexpr int kCoulI = 32;               // atoms per block
constexpr int kCoulJ = 16;               // positions per tile
constexpr int kCoulW = 8;                // pair warps (kCoulJ / kCoulW positions each per tile)
constexpr int kCoulThreads = 32 * (kCoulW + 1);

__global__ void __launch_bounds__(kCoulThreads) k_coulomb_allpairs(DevSys d, Params P) {
    __shared__ double jx[2][kCoulJ], jy[2][kCoulJ], jz[2][kCoulJ];
    __shared__ float jf[2][kCoulJ][3];    // float truncations of the positions (image test)
    __shared__ float jq[2][kCoulJ];
    __shared__ int jm[2][kCoulJ];
    __shared__ double tfx[2][kCoulJ][kCoulI], tfy[2][kCoulJ][kCoulI], tfz[2][kCoulJ][kCoulI];
    __shared__ float tu[2][kCoulJ][kCoulI];
    __shared__ unsigned ton[2][kCoulJ];   // bit a: the term of (atom a, position jj) is added
    if(d.sc->overflow) return;            // the step is redone after the neighbour list grows
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = P.n;
    const int k = blockIdx.x * kCoulI + lane;
    const bool live = k < n && d.mobile[k];
    const float qk = live ? d.qf[k] : 0.0f;
    if(!__syncthreads_or(qk != 0.0f)) return;
    const bool mine = qk != 0.0f;
    __shared__ BoxImage bx;
    if(threadIdx.x < 3) {
        const int a = threadIdx.x;
        const float Lf = box_f(d, P, a);
        const double w = double(Lf) / 2.0 - (-double(Lf) / 2.0);
        bx.w[a] = w;
        bx.nw[a] = -w;
        bx.hw[a] = __double_as_longlong(w / 2.0);
        bx.hwf[a] = __double2float_rn(w / 2.0);
    }
    const int ntile = (n + kCoulJ - 1) / kCoulJ;
    auto fetch = [&](int t, double& x, double& y, double& z, float& q, int& m) {
        const int j = t * kCoulJ + (int)threadIdx.x;
        if(j < n) {
            x = d.r[3 * j];
            y = d.r[3 * j + 1];
            z = d.r[3 * j + 2];
            q = d.qf[j];
            m = d.mol[j];
        }
    };
    auto park = [&](int b, double x, double y, double z, float q, int m) {
        jx[b][threadIdx.x] = x;
        jy[b][threadIdx.x] = y;
        jz[b][threadIdx.x] = z;
        jf[b][threadIdx.x][0] = trunc_f(x);
        jf[b][threadIdx.x][1] = trunc_f(y);
        jf[b][threadIdx.x][2] = trunc_f(z);
        jq[b][threadIdx.x] = q;
        jm[b][threadIdx.x] = m;
    };
    double sx = 0.0, sy = 0.0, sz = 0.0;
    float sq = 0.0f;
    int sm = -1;
    if(threadIdx.x < kCoulJ) {
        fetch(0, sx, sy, sz, sq, sm);
        park(0, sx, sy, sz, sq, sm);
    }
    if(warp < kCoulW) {
        // ---------------- pair warps ----------------
        const D3 rk = mine ? load3(d.r, k) : d3(0, 0, 0);
        const float rkf[3] = {trunc_f(rk.x), trunc_f(rk.y), trunc_f(rk.z)};
        const int molk = mine ? d.mol[k] : -1;
        const bool local = mine && d.excl_local[k] != 0;
        __syncthreads();
        for(int t = 0; t < ntile; t++) {
            const int b = t & 1;
            const bool stage = threadIdx.x < kCoulJ && t + 1 < ntile;
            if(stage) fetch(t + 1, sx, sy, sz, sq, sm);
#pragma unroll
            for(int h = 0; h < kCoulJ / kCoulW; h++) {
                const int jj = warp + h * kCoulW;
                const int j = t * kCoulJ + jj;
                bool on = false;
                D3 f = d3(0, 0, 0);
                float u = 0.0f;
                if(mine && j < n) {
                    const float qj = jq[b][jj];
                    if((kCoulombKf * qk * qj) != 0.0f) {
                        coulomb_pair(d, P, k, j, rk, d3(jx[b][jj], jy[b][jj], jz[b][jj]), rkf, jf[b][jj], qk, qj, molk,
                                     jm[b][jj], local, bx, f, u);
                        on = true;
                    }
                }
                const unsigned m = __ballot_sync(0xffffffffu, on);
                if(on) {
                    tfx[b][jj][lane] = f.x;
                    tfy[b][jj][lane] = f.y;
                    tfz[b][jj][lane] = f.z;
                    tu[b][jj][lane] = u;
                }
                if(lane == 0) ton[b][jj] = m;
            }
            if(stage) park(b ^ 1, sx, sy, sz, sq, sm);
            __syncthreads();
        }
        __syncthreads();   // the summing warp's last tile
    } else {
        // ---------------- summing warp: one tile behind ----------------
        double Fx = 0.0, Fy = 0.0, Fz = 0.0;
        float Uk = 0.0f;
        if(mine) {
            Fx = d.F[3 * k];
            Fy = d.F[3 * k + 1];
            Fz = d.F[3 * k + 2];
            Uk = (float)d.U[k];   // stored as double from a float: exact
        }
        __syncthreads();
        for(int t = 0; t <= ntile; t++) {
            if(t > 0) {
                const int b = (t - 1) & 1;
                const int m = min(kCoulJ, n - (t - 1) * kCoulJ);
                for(int jj = 0; jj < m; jj++) {
                    if((ton[b][jj] >> lane) & 1u) {
                        Fx += tfx[b][jj][lane];
                        Fy += tfy[b][jj][lane];
                        Fz += tfz[b][jj][lane];
                        Uk += tu[b][jj][lane];
                    }
                }
            }
            __syncthreads();
        }
        if(mine) {
            d.F[3 * k] = Fx;
            d.F[3 * k + 1] = Fy;
            d.F[3 * k + 2] = Fz;
            d.U[k] = (double)Uk;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Integration (VelVerlet.cpp:74-93 NVT/NVE branch, cutForces :96-122, pbcWrap SimulationBox.cpp:135-166)
// ---------------------------------------------------------------------------------------------
__global__ void k_kick_drift(DevSys d, Params P) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= P.n) return;
    const double S = d.sc->S;
    const double dt_2 = P.dt / 2.0;
    const double dm = P.dt / d.m[k];
#pragma unroll
    for(int a = 0; a < 3; a++) {
        double p = d.p[3 * k + a] * S;
        p = p + d.F[3 * k + a] * dt_2;
        d.p[3 * k + a] = p;
        d.r[3 * k + a] = d.r[3 * k + a] + p * dm;
    }
}

__device__ __forceinline__ double wrap_coord(double x, double Lm) {
    const double h = Lm / 2.0;
    if(x >= h) x -= double((int)((x + h) / Lm)) * Lm;
    if(x < -h) x -= double((int)((x + (-h)) / Lm)) * Lm;
    return x;
}

template<bool OUTPUT>
__global__ void k_kick2(DevSys d, Params P) {
    __shared__ double smem[32 * 3];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};   // sum p^2/m, sum F.r, sum U
    if(k < P.n) {
        const double dt_2 = P.dt / 2.0;
        double p2 = 0.0, fr = 0.0;
#pragma unroll
        for(int a = 0; a < 3; a++) {
            double f = d.F[3 * k + a];
            if(P.clip && P.fcut > 0.0 && fabs(f) > P.fcut) {
                f = ((f >= 0.0) ? 1.0 : -1.0) * P.fcut;
                d.F[3 * k + a] = f;
            }
            const double p = d.p[3 * k + a] + f * dt_2;
            d.p[3 * k + a] = p;
            const double x = wrap_coord(d.r[3 * k + a], P.box[a]);
            d.r[3 * k + a] = x;
            p2 += p * p;
            fr += f * x;
        }
        v[0] = p2 / d.m[k];
        if(OUTPUT) {
            v[1] = fr;
            v[2] = d.U[k];
        }
    }
    block_sum<3>(v, smem);
    if(threadIdx.x == 0) {
        d.partial[blockIdx.x * 4 + 0] = v[0];
        d.partial[blockIdx.x * 4 + 1] = v[1];
        d.partial[blockIdx.x * 4 + 2] = v[2];
    }
    if(last_block(&d.sc->done_blocks)) {
        __shared__ double tot[3];
        if(threadIdx.x == 0) {
            double s[3] = {0.0, 0.0, 0.0};
            for(int b = 0; b < (int)gridDim.x; b++)
                for(int q = 0; q < 3; q++) s[q] += d.partial[b * 4 + q];
            for(int q = 0; q < 3; q++) tot[q] = s[q];
            d.sc->done_blocks = 0;
        }
        __syncthreads();
        if(threadIdx.x < 96) {
            // the virial uses momenta after the thermostat: sum (c2 p)^2/m = c2^2 sum p^2/m,
            // folded in by end_of_step through KE2
            end_of_step<false>(P, d.sc, d.th, d.th_saved, tot[0], tot[2], tot[1], OUTPUT, d.rec);
        }
    }
}

// NPT branch (VelVerlet.cpp:57-71): steps 3.2 prop_p and 3.3 prop_r with the coefficients the
// previous step's last block derived from p_eps (3.1); momenta carry the pending thermostat scale.
__global__ void k_kick_drift_npt(DevSys d, Params P) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= P.n) return;
    const double S = d.sc->S;
    const BaroDev* b = d.baro;
    const double ap = b->ap, bp = b->bp, ar = b->ar, br = b->br;
    const double im = 1.0 / d.m[k];
#pragma unroll
    for(int a = 0; a < 3; a++) {
        double p = d.p[3 * k + a] * S;
        p = p * ap + d.F[3 * k + a] * bp;
        d.p[3 * k + a] = p;
        d.r[3 * k + a] = d.r[3 * k + a] * ar + (p * im) * br;
    }
}

// NPT: 3.5 prop_p with the new forces (no clipping in this branch), pbcWrap in the current box,
// and the sums sum p^2/m, sum F.r (unwrapped, for 3.6), sum F.r (wrapped, for 3.1 and P), sum U.
template<bool OUTPUT>
__global__ void k_kick2_npt(DevSys d, Params P) {
    __shared__ double smem[32 * 4];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if(k < P.n) {
        const BaroDev* b = d.baro;
        const double ap = b->ap, bp = b->bp;
        double p2 = 0.0, fu = 0.0, fw = 0.0;
#pragma unroll
        for(int a = 0; a < 3; a++) {
            const double f = d.F[3 * k + a];
            const double p = d.p[3 * k + a] * ap + f * bp;
            d.p[3 * k + a] = p;
            const double x0 = d.r[3 * k + a];
            const double x = wrap_coord(x0, b->L[a]);
            d.r[3 * k + a] = x;
            p2 += p * p;
            fu += f * x0;
            fw += f * x;
        }
        v[0] = p2 / d.m[k];
        v[1] = fu;
        v[2] = fw;
        if(OUTPUT) v[3] = d.U[k];
    }
    block_sum<4>(v, smem);
    if(threadIdx.x == 0) {
#pragma unroll
        for(int q = 0; q < 4; q++) d.partial[blockIdx.x * 4 + q] = v[q];
    }
    if(last_block(&d.sc->done_blocks)) {
        __shared__ double tot[4];
        if(threadIdx.x == 0) {
            double s[4] = {0.0, 0.0, 0.0, 0.0};
            for(int bk = 0; bk < (int)gridDim.x; bk++)
                for(int q = 0; q < 4; q++) s[q] += d.partial[bk * 4 + q];
            for(int q = 0; q < 4; q++) tot[q] = s[q];
            d.sc->done_blocks = 0;
        }
        __syncthreads();
        if(threadIdx.x < 96) npt_scalars<false>(P, d, tot[0], tot[1], tot[2], tot[3], true, OUTPUT);
    }
}

}  // namespace

// ---------------------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------------------
static inline int nblk(int n, int t) { return (n + t - 1) / t; }

void launch_ref_cells(const DevSys& d, const Params& P, cudaStream_t s) {
    const int ncell = P.nx * P.ny * P.nz;
    cudaMemsetAsync(d.cell_count, 0, sizeof(int) * ncell, s);
    k_cell_assign<<<nblk(P.n, 256), 256, 0, s>>>(d, P);
    k_cell_scan<<<1, 1024, 0, s>>>(d, ncell);
    // the scatter target doubles as scratch: nbr_count is rewritten by the neighbour kernel
    k_cell_scatter<<<nblk(P.n, 256), 256, 0, s>>>(d, P, d.nbr_count);
    k_cell_rank<<<nblk(ncell * 32, 256), 256, 0, s>>>(d, ncell, d.nbr_count);
}

void launch_ref_neigh(const DevSys& d, const Params& P, cudaStream_t s) {
    k_neigh<<<nblk(P.n * 32, 256), 256, 0, s>>>(d, P, P.rc);
}

void launch_ref_force(const DevSys& d, const Params& P, cudaStream_t s) {
    k_force<<<nblk(P.n, kRefTile), kRefTile, 0, s>>>(d, P);
    k_sr_parked<<<nblk(P.n, 32), 32 * (kSrW + 1), 0, s>>>(d, P);
    if(P.qany) k_coulomb_allpairs<<<nblk(P.n, kCoulI), kCoulThreads, 0, s>>>(d, P);
}

void launch_ref_kick_drift(const DevSys& d, const Params& P, cudaStream_t s) {
    if(P.ensemble == MTG_NPT) k_kick_drift_npt<<<nblk(P.n, 256), 256, 0, s>>>(d, P);
    else k_kick_drift<<<nblk(P.n, 256), 256, 0, s>>>(d, P);
}

void launch_ref_kick2(const DevSys& d, const Params& P, bool output, cudaStream_t s) {
    const int nb = reduction_blocks(P.n);
    if(P.ensemble == MTG_NPT) {
        if(output) k_kick2_npt<true><<<nb, 256, 0, s>>>(d, P);
        else k_kick2_npt<false><<<nb, 256, 0, s>>>(d, P);
        return;
    }
    if(output) k_kick2<true><<<nb, 256, 0, s>>>(d, P);
    else k_kick2<false><<<nb, 256, 0, s>>>(d, P);
}

}  // namespace mtg
