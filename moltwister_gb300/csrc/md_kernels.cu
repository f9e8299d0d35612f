// Production kernels: analytic force field in FP64 or mixed precision, Verlet neighbour list with
// a skin, fused integrator kernels, and the reduction/thermostat prologue shared by all modes.
//
// Layout in HBM (per atom):
//   FP64 mode : r double[3] (master), p double[3], F double[3]
//   mixed     : hi float4 (x,y,z hi, charge), lo float4 (x,y,z lo, type bits) -- the positions,
//               held as FP32 hi+lo pairs and updated in FP64 -- p double[3], F int64 x3 (SoA,
//               2^32 units per kJ/mol/A: per-pair contributions are rounded to fixed point and
//               summed exactly, so the result does not depend on summation order), inv_m float.
// Neighbour list: [atom][slot] uint32, atom index in the low 29 bits and the exclusion class of
// the pair (none, 1-2, 1-3, 1-4, same molecule; FunctorCalcForce.cpp:95-157) in the top 3 bits.
// Pairs whose class scale is exactly 0 are left out of the list.  Rebuilt when an atom has moved
// more than skin/2 since the last build.
//
// The force gather keeps the reference's structure (FunctorCalcForce.cpp:159-281): each atom sums
// its own bonded terms, its neighbours and (cutoff) Coulomb, using the full list, so no atomics are
// needed and the energy bookkeeping (pair energy on the lower index, angle energy on the centre,
// half the dihedral energy on each centre atom) is the reference's.
#include <float.h>
#include <stdint.h>

#include <cuda_device_runtime_api.h>

#include "md_device.cuh"
#include "mtg_internal.h"

namespace mtg {

int reduction_blocks(int n) {
    int b = (n + 255) / 256;
    return b < 1 ? 1 : b;
}

int integration_blocks(const Params& P) { return P.nrep ? P.nblk_total : reduction_blocks(P.n); }

namespace {

// The system an atom or an integration block belongs to: the whole context (r < 0), or replica r
// of a batch.  Gives the atom and block ranges, cell grid, box, cutoffs, temperature and the
// per-system scalars, chains and output record.
struct SysView {
    int off, n, bbase, nb;
    int cbase, pnx, pny, pnz;
    double box[3];
    double fconv[3];
    float fscale[3];
    float rc, rcoul, skin;
    double kT;
    StepScalars* sc;
    ThermoDev* th;
    ThermoDev* th_saved;
    double* rec;
};

__device__ __forceinline__ SysView sys_view(const DevSys& d, const Params& P, int r) {
    SysView v;
    if(r < 0) {
        v.off = 0; v.n = P.n; v.bbase = 0; v.nb = (P.n + 255) / 256;
        v.cbase = 0; v.pnx = P.pnx; v.pny = P.pny; v.pnz = P.pnz;
        for(int a = 0; a < 3; a++) {
            v.box[a] = P.box[a];
            v.fconv[a] = P.fconv[a];
            v.fscale[a] = P.fscale[a];
        }
        v.rc = P.rc; v.rcoul = P.rcoul; v.skin = P.skin; v.kT = P.kT;
        v.sc = d.sc; v.th = d.th; v.th_saved = d.th_saved; v.rec = d.rec;
    } else {
        const RepDev& R = d.reps[r];
        v.off = R.off; v.n = R.n; v.bbase = R.bbase; v.nb = R.nb;
        v.cbase = R.cbase; v.pnx = R.pnx; v.pny = R.pny; v.pnz = R.pnz;
        for(int a = 0; a < 3; a++) {
            v.box[a] = R.box[a];
            v.fconv[a] = R.fconv[a];
            v.fscale[a] = R.fscale[a];
        }
        v.rc = R.rc; v.rcoul = R.rcoul; v.skin = R.skin; v.kT = R.kT;
        v.sc = d.rsc + r; v.th = d.ths + r; v.th_saved = d.ths_saved + r; v.rec = d.rrec + 8 * r;
    }
    return v;
}

__device__ __forceinline__ int rep_of_atom(const DevSys& d, const Params& P, int i) { return P.nrep ? d.rep_of[i] : -1; }
__device__ __forceinline__ int rep_of_block(const DevSys& d, const Params& P) { return P.nrep ? d.blk_rep[blockIdx.x] : -1; }


// ---------------------------------------------------------------------------------------------
// Prologue: sum p^2/m, then the first thermostat half-step of the coming step.
// ---------------------------------------------------------------------------------------------
__global__ void k_prologue(DevSys d, Params P) {
    __shared__ double smem[32 * 2];
    const SysView sv = sys_view(d, P, rep_of_block(d, P));
    const int k = sv.off + (blockIdx.x - sv.bbase) * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};   // sum p^2/m, sum F.r (NPT: G_eps of the first step, VelVerlet.cpp:60)
    if(k < sv.off + sv.n) {
        const double px = d.p[3 * k], py = d.p[3 * k + 1], pz = d.p[3 * k + 2];
        v[0] = (px * px + py * py + pz * pz) / d.m[k];
        if(P.ensemble == MTG_NPT)
            v[1] = d.F[3 * k] * d.r[3 * k] + d.F[3 * k + 1] * d.r[3 * k + 1] + d.F[3 * k + 2] * d.r[3 * k + 2];
    }
    block_sum<2>(v, smem);
    if(threadIdx.x == 0) {
        d.partial[blockIdx.x * 4] = v[0];
        d.partial[blockIdx.x * 4 + 1] = v[1];
    }
    if(last_block_of(&sv.sc->done_blocks, (unsigned)sv.nb)) {
        __shared__ double tot, tot_fr;
        if(threadIdx.x == 0) {
            double KE2 = 0.0, fr = 0.0;
            for(int b = sv.bbase; b < sv.bbase + sv.nb; b++) {
                KE2 += d.partial[b * 4];
                fr += d.partial[b * 4 + 1];
            }
            tot = KE2;
            tot_fr = fr;
            sv.sc->done_blocks = 0;
        }
        __syncthreads();
        if(P.ensemble == MTG_NPT) {
            if(threadIdx.x < 96) npt_scalars(P, d, tot, 0.0, tot_fr, 0.0, false, false);
            if(threadIdx.x == 0) d.sc->c2 = 1.0;
            return;
        }
        if(threadIdx.x < 96) {
            double KE2 = tot;
            double c2 = 1.0, c1 = 1.0;
            Params Q = P;
            Q.n = sv.n;
            Q.kT = sv.kT;
            if(P.ensemble == MTG_NVT || P.ensemble == MTG_NPT) thermostat(Q, sv.sc, sv.th, sv.th_saved, KE2, false, &c2, &c1);
            if(threadIdx.x == 0) {
                sv.sc->S = c1;
                sv.sc->c2 = 1.0;
                if(sv.sc->timeout) d.sc->timeout = 1;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Position access
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void load_pos(const DevSys& d, int i, double& x, double& y, double& z, bool mixed) {
    if(mixed) {
        const float4 h = d.hi[i], l = d.lo[i];
        x = double(h.x) + double(l.x);
        y = double(h.y) + double(l.y);
        z = double(h.z) + double(l.z);
    } else {
        x = d.r[3 * i];
        y = d.r[3 * i + 1];
        z = d.r[3 * i + 2];
    }
}

// 32-bit fraction of the box: round(x / L * 2^32) modulo 2^32.  The difference of two such
// coordinates, read as a signed 32-bit integer, is the minimum-image separation in units of
// L / 2^32, exact for any |dx| < L/2 (no cancellation at the periodic boundary).
__device__ __forceinline__ unsigned int frac32(double x, double conv) {
    return (unsigned int)(unsigned long long)__double2ll_rn(x * conv);
}

__device__ __forceinline__ void store_pos(const DevSys& d, const double* conv, int i, double x, double y, double z,
                                          bool mixed) {
    if(mixed) {
        const float hx = (float)x, hy = (float)y, hz = (float)z;
        float4 h = d.hi[i], l = d.lo[i];
        h.x = hx; h.y = hy; h.z = hz;
        l.x = (float)(x - double(hx));
        l.y = (float)(y - double(hy));
        l.z = (float)(z - double(hz));
        d.hi[i] = h;
        d.lo[i] = l;
        uint4 q = d.pq[i];
        q.x = frac32(x, conv[0]);
        q.y = frac32(y, conv[1]);
        q.z = frac32(z, conv[2]);
        d.pq[i] = q;
    } else {
        d.r[3 * i] = x;
        d.r[3 * i + 1] = y;
        d.r[3 * i + 2] = z;
    }
}

__device__ __forceinline__ void load_force(const DevSys& d, int i, double& fx, double& fy, double& fz, bool mixed) {
    if(mixed) {
        fx = double(d.Fx[i]) * (1.0 / kFixScale);
        fy = double(d.Fy[i]) * (1.0 / kFixScale);
        fz = double(d.Fz[i]) * (1.0 / kFixScale);
    } else {
        fx = d.F[3 * i];
        fy = d.F[3 * i + 1];
        fz = d.F[3 * i + 2];
    }
}

// ---------------------------------------------------------------------------------------------
// Integration
// ---------------------------------------------------------------------------------------------
template<bool MIXED>
__device__ __forceinline__ void kick_drift_atom(DevSys& d, const Params& P, const SysView& v, int k);

// One 256-atom block per launch block; a batch maps blocks to replicas (blk_rep).
template<bool MIXED>
__global__ void k_pkick_drift(DevSys d, Params P, cudaGraphConditionalHandle cond) {
    const SysView v = sys_view(d, P, rep_of_block(d, P));
    const int k = v.off + (blockIdx.x - v.bbase) * blockDim.x + threadIdx.x;
    const bool mine = k < v.off + v.n;
    if(cond) {
        // inside a captured step graph: the last block hands the grid-wide rebuild decision to the
        // graph's IF node that wraps the list build
        if(mine) kick_drift_atom<MIXED>(d, P, v, k);
        if(last_block(&d.sc->done_blocks)) {
            if(threadIdx.x == 0) {
                d.sc->done_blocks = 0;
                cudaGraphSetConditional(cond, d.sc->rebuild ? 1u : 0u);
            }
        }
        return;
    }
    if(!mine) return;
    kick_drift_atom<MIXED>(d, P, v, k);
}

template<bool MIXED>
__device__ __forceinline__ void kick_drift_atom(DevSys& d, const Params& P, const SysView& v, int k) {
    const double S = v.sc->S;
    const double dt_2 = P.dt / 2.0;
    const double dm = P.dt / d.m[k];
    double fx, fy, fz, x, y, z;
    load_force(d, k, fx, fy, fz, MIXED);
    load_pos(d, k, x, y, z, MIXED);
    double px = d.p[3 * k] * S + fx * dt_2;
    double py = d.p[3 * k + 1] * S + fy * dt_2;
    double pz = d.p[3 * k + 2] * S + fz * dt_2;
    d.p[3 * k] = px;
    d.p[3 * k + 1] = py;
    d.p[3 * k + 2] = pz;
    x += px * dm;
    y += py * dm;
    z += pz * dm;
    store_pos(d, v.fconv, k, x, y, z, MIXED);
    // displacement since the last list build (minimum image: wrapping is not a displacement)
    const double bx = minimg_d(x - d.r_build[3 * k], v.box[0], 1.0 / v.box[0]);
    const double by = minimg_d(y - d.r_build[3 * k + 1], v.box[1], 1.0 / v.box[1]);
    const double bz = minimg_d(z - d.r_build[3 * k + 2], v.box[2], 1.0 / v.box[2]);
    const double h = 0.5 * double(v.skin);
    if(bx * bx + by * by + bz * bz > h * h) d.sc->rebuild = 1;
}

__device__ __forceinline__ double wrap_coord(double x, double Lm) {
    // pbcWrap (SimulationBox.cpp:135-166)
    const double h = Lm / 2.0;
    if(x >= h) x -= double((int)((x + h) / Lm)) * Lm;
    if(x < -h) x -= double((int)((x + (-h)) / Lm)) * Lm;
    return x;
}

template<bool MIXED, bool OUTPUT>
__global__ void k_pkick2(DevSys d, Params P) {
    __shared__ double smem[32 * 3];
    const SysView sv = sys_view(d, P, rep_of_block(d, P));
    const int k = sv.off + (blockIdx.x - sv.bbase) * blockDim.x + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    if(k < sv.off + sv.n) {
        const double dt_2 = P.dt / 2.0;
        double f[3], r[3];
        load_force(d, k, f[0], f[1], f[2], MIXED);
        load_pos(d, k, r[0], r[1], r[2], MIXED);
        double p2 = 0.0, fr = 0.0;
#pragma unroll
        for(int a = 0; a < 3; a++) {
            if(P.clip && P.fcut > 0.0 && fabs(f[a]) > P.fcut) {
                f[a] = ((f[a] >= 0.0) ? 1.0 : -1.0) * P.fcut;
                if(MIXED) {
                    long long q = (long long)(f[a] * kFixScale);
                    if(a == 0) d.Fx[k] = q; else if(a == 1) d.Fy[k] = q; else d.Fz[k] = q;
                } else {
                    d.F[3 * k + a] = f[a];
                }
            }
            const double p = d.p[3 * k + a] + f[a] * dt_2;
            d.p[3 * k + a] = p;
            r[a] = wrap_coord(r[a], sv.box[a]);
            p2 += p * p;
            fr += f[a] * r[a];
        }
        store_pos(d, sv.fconv, k, r[0], r[1], r[2], MIXED);
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
    if(last_block_of(&sv.sc->done_blocks, (unsigned)sv.nb)) {
        __shared__ double tot[3];
        if(threadIdx.x == 0) {
            double s[3] = {0.0, 0.0, 0.0};
            for(int b = sv.bbase; b < sv.bbase + sv.nb; b++)
                for(int q = 0; q < 3; q++) s[q] += d.partial[b * 4 + q];
            for(int q = 0; q < 3; q++) tot[q] = s[q];
            sv.sc->done_blocks = 0;
        }
        __syncthreads();
        if(threadIdx.x < 96) {
            if(P.nrep) {
                Params Q = P;   // the replica's size, temperature and box
                Q.n = sv.n;
                Q.kT = sv.kT;
                for(int a = 0; a < 3; a++) Q.box[a] = sv.box[a];
                end_of_step(Q, sv.sc, sv.th, sv.th_saved, tot[0], tot[2], tot[1], OUTPUT, sv.rec);
                if(threadIdx.x == 0 && sv.sc->timeout) d.sc->timeout = 1;
            } else {
                end_of_step(P, d.sc, d.th, d.th_saved, tot[0], tot[2], tot[1], OUTPUT, d.rec);
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Verlet list build: cell grid with edge >= rlist (or one cell for small boxes), counting sort
// with a per-cell rank pass (deterministic order), then one warp per atom scanning the 27 cells.
// ---------------------------------------------------------------------------------------------
template<bool MIXED>
__global__ void k_pcell_assign(DevSys d, Params P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n || !d.sc->rebuild) return;
    double x, y, z;
    load_pos(d, i, x, y, z, MIXED);
    d.r_build[3 * i] = x;
    d.r_build[3 * i + 1] = y;
    d.r_build[3 * i + 2] = z;
    d.rb4[i] = make_float4((float)x, (float)y, (float)z, 0.0f);
    const SysView v = sys_view(d, P, rep_of_atom(d, P, i));
    int ix = (int)floor((x + 0.5 * v.box[0]) * v.pnx / v.box[0]);
    int iy = (int)floor((y + 0.5 * v.box[1]) * v.pny / v.box[1]);
    int iz = (int)floor((z + 0.5 * v.box[2]) * v.pnz / v.box[2]);
    ix = ix < 0 ? 0 : (ix >= v.pnx ? v.pnx - 1 : ix);
    iy = iy < 0 ? 0 : (iy >= v.pny ? v.pny - 1 : iy);
    iz = iz < 0 ? 0 : (iz >= v.pnz ? v.pnz - 1 : iz);
    const int c = v.cbase + ix + v.pnx * (iy + v.pny * iz);
    d.pcell_of[i] = c;
    atomicAdd(&d.pcell_count[c], 1);
}

__global__ void k_pcell_scan(DevSys d, int ncell) {
    if(!d.sc->rebuild) return;
    __shared__ int warp_tot[32];
    __shared__ int carry;
    if(threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for(int base = 0; base < ncell; base += blockDim.x) {
        const int c = base + threadIdx.x;
        const int v = (c < ncell) ? d.pcell_count[c] : 0;
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
            d.pcell_first[c] = excl;
            d.pcell_cursor[c] = 0;
        }
        __syncthreads();
        if(threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
}

__global__ void k_pcell_scatter(DevSys d, Params P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n || !d.sc->rebuild) return;
    const int c = d.pcell_of[i];
    const int slot = atomicAdd(&d.pcell_cursor[c], 1);
    d.vcount[d.pcell_first[c] + slot] = i;   // vcount doubles as scratch until the list kernel
}

__global__ void k_pcell_rank(DevSys d, int ncell) {
    if(!d.sc->rebuild) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if(warp >= ncell) return;
    const int cnt = d.pcell_count[warp], first = d.pcell_first[warp];
    const int* tmp = d.vcount;
    for(int a = lane; a < cnt; a += 32) {
        const int v = tmp[first + a];
        int rank = 0;
        for(int b = 0; b < cnt; b++) rank += (tmp[first + b] < v);
        d.pcell_list[first + rank] = v;
    }
}

// Exclusion class of the pair (k, i) from k's bonded lists and molecule indices.
__device__ __forceinline__ int excl_class(const DevSys& d, int k, int i) {
    for(int e = d.bptr[k]; e < d.bptr[k + 1]; e++) if(d.bj[e] == i) return 1;
    for(int e = d.aptr[k]; e < d.aptr[k + 1]; e++) if(!d.acen[e] && d.aj[e] == i) return 2;
    for(int e = d.dptr[k]; e < d.dptr[k + 1]; e++) if(!d.dcen[e] && d.dl[e] == i) return 3;
    const int mi = d.mol[i], mk = d.mol[k];
    if(mi >= 0 && mk >= 0 && mi == mk) return 4;
    return 0;
}

template<bool MIXED>
__global__ void k_vlist(DevSys d, Params P) {
    if(!d.sc->rebuild) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if(i >= P.n) return;
    const SysView v = sys_view(d, P, rep_of_atom(d, P, i));
    const float rlist = fmaxf(v.rc, P.coulomb != MTG_COULOMB_ALLPAIRS ? v.rcoul : 0.0f) + v.skin;
    // FP32 distances: rounding (~1e-6 A) is far inside the skin margin
    const float4 ri = d.rb4[i];
    const float rl2 = rlist * rlist;
    const float Lx = (float)v.box[0], Ly = (float)v.box[1], Lz = (float)v.box[2];
    const float iLx = 1.0f / Lx, iLy = 1.0f / Ly, iLz = 1.0f / Lz;
    const int ci = d.pcell_of[i] - v.cbase;
    const int cx = ci % v.pnx, cy = (ci / v.pnx) % v.pny, cz = ci / (v.pnx * v.pny);
    const int sx = v.pnx >= 3 ? 3 : 1, sy = v.pny >= 3 ? 3 : 1, sz = v.pnz >= 3 ? 3 : 1;
    uint32_t* out = d.vlist + (size_t)i * d.vmax;
    int cnt = 0;
    for(int oz = 0; oz < sz; oz++) {
        const int z = sz == 1 ? 0 : (cz + oz - 1 + v.pnz) % v.pnz;
        for(int oy = 0; oy < sy; oy++) {
            const int y = sy == 1 ? 0 : (cy + oy - 1 + v.pny) % v.pny;
            for(int ox = 0; ox < sx; ox++) {
                const int x = sx == 1 ? 0 : (cx + ox - 1 + v.pnx) % v.pnx;
                const int c = v.cbase + x + v.pnx * (y + v.pny * z);
                const int first = d.pcell_first[c], n = d.pcell_count[c];
                for(int base = 0; base < n; base += 32) {
                    bool take = false;
                    uint32_t entry = 0;
                    if(base + lane < n) {
                        const int j = d.pcell_list[first + base + lane];
                        if(j != i) {
                            const float4 rj = d.rb4[j];
                            const float dx = minimg_f(ri.x - rj.x, Lx, iLx);
                            const float dy = minimg_f(ri.y - rj.y, Ly, iLy);
                            const float dz = minimg_f(ri.z - rj.z, Lz, iLz);
                            if(dx * dx + dy * dy + dz * dz < rl2) {
                                const int cls = excl_class(d, i, j);
                                if(P.scale[cls] != 0.0f) {
                                    take = true;
                                    entry = (uint32_t)j | ((uint32_t)cls << kClassShift);
                                }
                            }
                        }
                    }
                    const unsigned ball = __ballot_sync(0xffffffffu, take);
                    if(take) {
                        const int slot = cnt + __popc(ball & ((1u << lane) - 1u));
                        if(slot < d.vmax) out[slot] = entry;
                    }
                    cnt += __popc(ball);
                }
            }
        }
    }
    if(lane == 0) {
        d.vcount[i] = cnt;
        if(cnt > d.vmax) {
            d.sc->overflow = 1;
            atomicMax(&d.sc->needed, cnt);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Force gather
// ---------------------------------------------------------------------------------------------
template<class R>
struct Acc {
    R x, y, z;
};

// Fixed-point accumulation of FP32 contributions (mixed mode) without the FP64 unit.
// A contribution f becomes round(f * 2^26) exactly, split over two int32 accumulators:
//   h += round(f * 2^4)                  (adding 1.5 * 2^23 rounds a float of magnitude < 2^22 to an
//   l += round((f * 2^4 - h_i) * 2^22)    integer held in the low mantissa bits)
// and the lane's total is h * 2^22 + l in units of 2^-26 kJ/(mol A).  Every step is exact in FP32,
// so the fixed-point value of each contribution, and hence every sum of them, is independent of
// the order of summation.  |f| is clamped to 2^18 (no physical pair force comes near it).
struct Fix {
    int h, l;
};
__device__ __forceinline__ void fix_add(Fix& a, float f) {
    const float M = 12582912.0f;                 // 1.5 * 2^23
    const float x = __fmul_rn(f, 16.0f);
    const float tx = __fadd_rn(x, M);
    const float rx = __fsub_rn(x, __fsub_rn(tx, M));
    a.h += __float_as_int(tx) - __float_as_int(M);
    const float ty = __fadd_rn(__fmul_rn(rx, 4194304.0f), M);
    a.l += __float_as_int(ty) - __float_as_int(M);
}
__device__ __forceinline__ void fix_add_clamped(Fix& a, float f) { fix_add(a, fminf(fmaxf(f, -262143.0f), 262143.0f)); }
__device__ __forceinline__ long long fix_total(const Fix& a) { return ((long long)a.h << 22) + (long long)a.l; }

// -dU/dr / r (= g) and U of the analytic pair terms for type pair `pair`; table kinds interpolate.
// ir2 = 1/r^2 and ir = 1/r are passed in (rsqrt in FP32).
template<class R>
__device__ __forceinline__ void pair_terms(const DevSys& d, int pair, R r2, R ir, R ir2, R& g, R& u, bool energy,
                                           int P_lj_shift) {
    const int cnt = d.nb_cnt[pair];
    for(int ff = 0; ff < cnt; ff++) {
        const int idx = pair * kMaxFF + ff;
        const int kind = d.nb_kind[idx];
        R a, b, c, dd;
        if(sizeof(R) == 4) {
            const float4 q = reinterpret_cast<const float4*>(d.nb_parf)[idx];
            a = (R)q.x; b = (R)q.y; c = (R)q.z; dd = (R)q.w;
        } else {
            a = (R)d.nb_par[4 * idx]; b = (R)d.nb_par[4 * idx + 1]; c = (R)d.nb_par[4 * idx + 2];
            dd = (R)d.nb_par[4 * idx + 3];
        }
        if(kind == MTG_NB_LJ) {
            // a = 4 eps sigma^12, b = 4 eps alpha sigma^6, c = own cutoff^2 (0: global), d = energy
            // shift; force-shifted LJ also subtracts F(rc) (fs) and adds r F(rc) to the energy
            if(c == R(0) || r2 < c) {
                const R ir6 = ir2 * ir2 * ir2;
                const R t12 = a * ir6 * ir6, t6 = b * ir6;
                g += (R(12) * t12 - R(6) * t6) * ir2;
                if(energy) u += t12 - t6 - dd;
                if(P_lj_shift == 2) {
                    const R fs = sizeof(R) == 4 ? (R)d.nb_fsf[idx] : (R)d.nb_fs[idx];
                    g -= fs * ir;
                    if(energy) u += r2 * ir * fs;
                }
            }
        } else if(kind == MTG_NB_LJ1208) {
            if(c == R(0) || r2 < c) {
                const R ir4 = ir2 * ir2, ir8 = ir4 * ir4;
                const R t12 = a * ir8 * ir4, t8 = b * ir8;
                g += (R(12) * t12 - R(8) * t8) * ir2;
                if(energy) u += t12 - t8 - dd;
                if(P_lj_shift == 2) {
                    const R fs = sizeof(R) == 4 ? (R)d.nb_fsf[idx] : (R)d.nb_fs[idx];
                    g -= fs * ir;
                    if(energy) u += r2 * ir * fs;
                }
            }
        } else if(kind == MTG_NB_BUCK) {
            // a = A, b = 1/rho, c = C
            const R r = r2 * ir;
            const R ir6 = ir2 * ir2 * ir2;
            const R e = a * exp(-r * b);
            g += e * b * ir - R(6) * c * ir6 * ir2;
            if(energy) u += e - c * ir6;
        } else {
            // tabulated kind: linear interpolation of (x, -dU/dx, U) like the reference
            const float* tab = d.nb_tab + (size_t)idx * kNpts * 3;
            const float rr = (float)(r2 * ir);
            const float delta = (tab[3 * (kNpts - 1)] - tab[0]) / float(kNpts - 1);
            const float q = (rr - tab[0]) / delta;
            if(q >= 0.0f && q < float(kNpts - 1)) {
                const int t = (int)q;
                const float* p1 = tab + 3 * t;
                const float* p2 = p1 + 3;
                const float sl = (p1[1] - p2[1]) / (p1[0] - p2[0]);
                g += R((sl * rr + (p1[1] - sl * p1[0])) / rr);
                if(energy) {
                    const float ae = (p1[2] - p2[2]) / (p1[0] - p2[0]);
                    u += R(ae * rr + (p1[2] - ae * p1[0]));
                }
            }
        }
    }
}

// Relative vector r_i - r_j (minimum image) in the arithmetic precision R.
template<bool MIXED, class R>
__device__ __forceinline__ void rel(const DevSys& d, const Params& P, int i, int j, R& dx, R& dy, R& dz) {
    const SysView v = sys_view(d, P, rep_of_atom(d, P, i));
    if(MIXED) {
        const uint4 qi = d.pq[i], qj = d.pq[j];
        dx = (R)__int2float_rn((int)(qi.x - qj.x)) * (R)v.fscale[0];
        dy = (R)__int2float_rn((int)(qi.y - qj.y)) * (R)v.fscale[1];
        dz = (R)__int2float_rn((int)(qi.z - qj.z)) * (R)v.fscale[2];
    } else {
        dx = (R)minimg_d(d.r[3 * i] - d.r[3 * j], v.box[0], 1.0 / v.box[0]);
        dy = (R)minimg_d(d.r[3 * i + 1] - d.r[3 * j + 1], v.box[1], 1.0 / v.box[1]);
        dz = (R)minimg_d(d.r[3 * i + 2] - d.r[3 * j + 2], v.box[2], 1.0 / v.box[2]);
    }
}

template<class R>
__device__ __forceinline__ R acos_clamped(R c) {
    c = c > R(1) ? R(1) : (c < R(-1) ? R(-1) : c);
    return acos(c);
}

template<class R>
__device__ __forceinline__ void load_par(const double* pd, const float* pf, int t, R (&p)[4]) {
    if(sizeof(R) == 4) {
        const float4 q = reinterpret_cast<const float4*>(pf)[t];
        p[0] = (R)q.x; p[1] = (R)q.y; p[2] = (R)q.z; p[3] = (R)q.w;
    } else {
        for(int w = 0; w < 4; w++) p[w] = (R)pd[4 * t + w];
    }
}

// Bonded contribution of entry `e` (global bonded-entry index space: bonds, then angles, then
// dihedrals of atom k) to the force on k, and to k's energy (reference bookkeeping).
template<bool MIXED, class R>
__device__ void bonded_entry(const DevSys& d, const Params& P, int k, int e, R& fx, R& fy, R& fz, R& u, bool energy) {
    const int nb = d.bptr[k + 1] - d.bptr[k];
    const int na = d.aptr[k + 1] - d.aptr[k];
    if(e < nb) {
        const int q = d.bptr[k] + e;
        const int i = d.bj[q], t = d.bt[q];
        R dx, dy, dz;
        rel<MIXED, R>(d, P, k, i, dx, dy, dz);     // r_k - r_i
        const R r = sqrt(dx * dx + dy * dy + dz * dz);
        const int kind = d.bond_kind[t];
        R md = 0, uu = 0;
        R p[4];
        load_par<R>(d.bond_par, d.bond_parf, t, p);
        if(kind == MTG_BOND_HARM) {
            const R dr = r - (R)p[1];
            md = -R(2) * (R)p[0] * dr;
            uu = (R)p[0] * dr * dr;
        } else if(kind == MTG_BOND_MORSE) {
            const R ex = exp(-(R)p[1] * (r - (R)p[2]));
            md = -R(2) * (R)p[0] * (R)p[1] * ex * (R(1) - ex);
            uu = (R)p[0] * (R(1) - ex) * (R(1) - ex);
        } else {
            const float* tab = d.bond_tab + (size_t)t * kNpts * 3;
            const float rr = (float)r;
            const float delta = (tab[3 * (kNpts - 1)] - tab[0]) / float(kNpts - 1);
            const float qq = (rr - tab[0]) / delta;
            if(qq >= 0.0f && qq < float(kNpts - 1)) {
                const int ti = (int)qq;
                const float* p1 = tab + 3 * ti;
                const float* p2 = p1 + 3;
                const float a = (p1[1] - p2[1]) / (p1[0] - p2[0]);
                md = R(a * rr + (p1[1] - a * p1[0]));
                const float ae = (p1[2] - p2[2]) / (p1[0] - p2[0]);
                uu = R(ae * rr + (p1[2] - ae * p1[0]));
            }
        }
        const R s = md / r;
        fx += s * dx; fy += s * dy; fz += s * dz;
        if(energy && i > k) u += uu;
        return;
    }
    e -= nb;
    if(e < na) {
        const int q = d.aptr[k] + e;
        const int t = d.at[q];
        int c, a1, a3;
        if(d.acen[q]) { c = k; a1 = d.ai[q]; a3 = d.aj[q]; }
        else { c = d.ai[q]; a1 = k; a3 = d.aj[q]; }
        R ux, uy, uz, vx, vy, vz;
        rel<MIXED, R>(d, P, a1, c, ux, uy, uz);
        rel<MIXED, R>(d, P, a3, c, vx, vy, vz);
        const R n1 = sqrt(ux * ux + uy * uy + uz * uz), n3 = sqrt(vx * vx + vy * vy + vz * vz);
        const R cs = (ux * vx + uy * vy + uz * vz) / (n1 * n3);
        const R th = acos_clamped(cs);
        R sn = sqrt(R(1) - cs * cs);
        sn = sn < R(1e-6) ? R(1e-6) : sn;
        R p[4];
        load_par<R>(d.angle_par, d.angle_parf, t, p);   // (k, theta0 [rad], toRad, 0)
        R dU = 0, uu = 0;
        if(d.angle_kind[t] == MTG_ANGLE_HARM) {
            const R dd = th - p[1];
            dU = R(2) * (R)p[0] * dd;
            uu = (R)p[0] * dd * dd;
        } else {
            // tabulated: the table holds -dU/dtheta
            const float* tab = d.angle_tab + (size_t)t * kNpts * 3;
            const float tt = (float)th;
            const float delta = (tab[3 * (kNpts - 1)] - tab[0]) / float(kNpts - 1);
            const float qq = (tt - tab[0]) / delta;
            if(qq >= 0.0f && qq < float(kNpts - 1)) {
                const int ti = (int)qq;
                const float* p1 = tab + 3 * ti;
                const float* p2 = p1 + 3;
                const float a = (p1[1] - p2[1]) / (p1[0] - p2[0]);
                dU = -R(a * tt + (p1[1] - a * p1[0]));
                const float ae = (p1[2] - p2[2]) / (p1[0] - p2[0]);
                uu = R(ae * tt + (p1[2] - ae * p1[0]));
            }
        }
        // d theta / d u = -(v/(n1 n3) - cs u / n1^2) / sin, similarly for v
        const R inv = R(1) / (n1 * n3);
        const R g1x = -(vx * inv - cs * ux / (n1 * n1)) / sn, g1y = -(vy * inv - cs * uy / (n1 * n1)) / sn,
                g1z = -(vz * inv - cs * uz / (n1 * n1)) / sn;
        if(d.acen[q]) {
            const R g3x = -(ux * inv - cs * vx / (n3 * n3)) / sn, g3y = -(uy * inv - cs * vy / (n3 * n3)) / sn,
                    g3z = -(uz * inv - cs * vz / (n3 * n3)) / sn;
            fx += dU * (g1x + g3x); fy += dU * (g1y + g3y); fz += dU * (g1z + g3z);
            if(energy) u += uu;
        } else {
            fx -= dU * g1x; fy -= dU * g1y; fz -= dU * g1z;
        }
        return;
    }
    e -= na;
    {
        const int q = d.dptr[k] + e;
        const int t = d.dt[q];
        int a, b, c, dd;
        if(d.dcen[q]) { a = d.di[q]; b = k; c = d.dj[q]; dd = d.dl[q]; }
        else { a = k; b = d.di[q]; c = d.dj[q]; dd = d.dl[q]; }
        R b1x, b1y, b1z, b2x, b2y, b2z, b3x, b3y, b3z;
        rel<MIXED, R>(d, P, b, a, b1x, b1y, b1z);
        rel<MIXED, R>(d, P, c, b, b2x, b2y, b2z);
        rel<MIXED, R>(d, P, dd, c, b3x, b3y, b3z);
        const R mx = b1y * b2z - b1z * b2y, my = b1z * b2x - b1x * b2z, mz = b1x * b2y - b1y * b2x;
        const R nx = b2y * b3z - b2z * b3y, ny = b2z * b3x - b2x * b3z, nz = b2x * b3y - b2y * b3x;
        const R m2 = mx * mx + my * my + mz * mz, n2 = nx * nx + ny * ny + nz * nz;
        const R lb2 = sqrt(b2x * b2x + b2y * b2y + b2z * b2z);
        if(!(m2 > R(1e-20) && n2 > R(1e-20))) return;
        const R cs = (mx * nx + my * ny + mz * nz) / sqrt(m2 * n2);
        const R phi = acos_clamped(cs);
        R p[4];
        load_par<R>(d.dih_par, d.dih_parf, t, p);
        const int kind = d.dih_kind[t];
        R dV = 0, V = 0;
        if(kind == MTG_DIH_HARM) {
            const R K = (R)p[0];
            const int D = (int)p[1], N = (int)p[2];
            dV = -K * R(D * N) * sin(R(N) * phi);
            V = K * (R(1) + R(D) * cos(R(N) * phi));
        } else if(kind == MTG_DIH_FOURIER4T) {
            dV = R(-0.5) * (R)p[0] * sin(phi) + (R)p[1] * sin(R(2) * phi) + R(-1.5) * (R)p[2] * sin(R(3) * phi) +
                 R(2) * (R)p[3] * sin(R(4) * phi);
            V = R(0.5) * ((R)p[0] * (R(1) + cos(phi)) + (R)p[1] * (R(1) - cos(R(2) * phi)) +
                          (R)p[2] * (R(1) + cos(R(3) * phi)) + (R)p[3] * (R(1) - cos(R(4) * phi)));
        }
        // gradient of the signed dihedral; |psi| = phi, sign = sign(b1 . n)
        const R sgn = (b1x * nx + b1y * ny + b1z * nz) >= R(0) ? R(1) : R(-1);
        const R ga = -lb2 / m2, gd = lb2 / n2;
        R gx, gy, gz;
        if(d.dcen[q]) {
            const R f1 = (b1x * b2x + b1y * b2y + b1z * b2z) / (lb2 * lb2);
            const R f3 = (b3x * b2x + b3y * b2y + b3z * b2z) / (lb2 * lb2);
            gx = -(R(1) + f1) * ga * mx + f3 * gd * nx;
            gy = -(R(1) + f1) * ga * my + f3 * gd * ny;
            gz = -(R(1) + f1) * ga * mz + f3 * gd * nz;
            if(energy) u += R(0.5) * V;
        } else {
            gx = ga * mx; gy = ga * my; gz = ga * mz;
        }
        fx -= dV * sgn * gx; fy -= dV * sgn * gy; fz -= dV * sgn * gz;
    }
}

// One neighbour-list entry of atom i: force factor g (F_i += g * d) and pair energy u.
// Per type pair, staged in shared memory by the force kernel: mode 0 = no term, 1 = one 12-6 LJ
// term with coefficients (a, b), 2 = anything else (evaluated by pair_terms from global memory).
struct PairCoef {
    float a, b;       // 4 eps sigma^12, 4 eps alpha sigma^6
    float rc2, us;    // own cutoff^2 (0: global), energy shift
    float fs, pad0, pad1, pad2;   // force at the cutoff (force-shifted LJ)
};
constexpr int kSmemPairs = 64;   // type pairs staged (T <= 8)

template<bool MIXED, bool ENERGY, class R>
__device__ __forceinline__ void pair_entry(const DevSys& d, const Params& P, int i, uint32_t ent, int ti, R qi,
                                           R rc2, R rq2, R irc, R kq, const PairCoef* pc, const int* pmode,
                                           const float* qt, uint4 qi4, const float (&fs)[3], R& dx, R& dy, R& dz,
                                           R& g, R& u) {
    const int j = (int)(ent & kIdxMask);
    const int cls = (int)(ent >> kClassShift);
    int tj;
    if(MIXED) {
        const uint4 qj4 = d.pq[j];
        dx = (R)__int2float_rn((int)(qi4.x - qj4.x)) * (R)fs[0];
        dy = (R)__int2float_rn((int)(qi4.y - qj4.y)) * (R)fs[1];
        dz = (R)__int2float_rn((int)(qi4.z - qj4.z)) * (R)fs[2];
        tj = (int)qj4.w;
    } else {
        rel<MIXED, R>(d, P, i, j, dx, dy, dz);
        tj = d.type[j];
    }
    const R r2 = dx * dx + dy * dy + dz * dz;
    R ir;
    if(MIXED) ir = (R)rsqrtf((float)r2);
    else ir = R(1) / sqrt(r2);
    const R ir2 = ir * ir;
    g = 0;
    u = 0;
    if(r2 < rc2 && r2 >= R(1e-6)) {
        const int pr = ti * P.T + tj;
        if(MIXED && pc && pr < kSmemPairs) {
            const int mode = pmode[pr];
            if(mode == 1) {
                const PairCoef c = pc[pr];
                if(c.rc2 == 0.0f || (float)r2 < c.rc2) {
                    const R ir6 = ir2 * ir2 * ir2;
                    const R t12 = (R)c.a * ir6 * ir6, t6 = (R)c.b * ir6;
                    g = (R(12) * t12 - R(6) * t6) * ir2 - (R)c.fs * ir;
                    if(ENERGY) u = t12 - t6 - (R)c.us + r2 * ir * (R)c.fs;
                }
            } else if(mode == 2) {
                pair_terms<R>(d, pr, r2, ir, ir2, g, u, ENERGY, P.lj_shift);
            }
        } else {
            pair_terms<R>(d, pr, r2, ir, ir2, g, u, ENERGY, P.lj_shift);
        }
    }
    if(P.coulomb != MTG_COULOMB_ALLPAIRS && r2 < rq2) {
        const R qj = MIXED ? (R)(qt ? qt[tj] : d.qf[j]) : (R)d.qd[j];
        const R qq = kq * qi * qj;
        if(P.coulomb == MTG_COULOMB_SHIFTED) {
            g += qq * (ir2 - irc * irc) * ir;
            if(ENERGY) u += qq * (ir - irc + (r2 * ir - R(1) / irc) * irc * irc);
        } else {
            g += qq * ir2 * ir;
            if(ENERGY) u += qq * ir;
        }
    }
    if(cls) {
        const R sc = (R)P.scale[cls];
        g *= sc;
        u *= sc;
    }
    if(!(ENERGY && j > i)) u = 0;
}

// Force gather: TEAM lanes per atom (8, 16 or 32; chosen per system by the autotuner), each lane
// walking its share of the atom's neighbour-list row four entries at a time so that four gathers
// are in flight per lane.  Bonded terms of the atom are spread over the team's lanes.
template<bool MIXED, bool ENERGY, int TEAM>
__global__ void __launch_bounds__(256, 4) k_pforce(DevSys d, Params P) {
    using R = typename std::conditional<MIXED, float, double>::type;
    __shared__ PairCoef pc_s[kSmemPairs];
    __shared__ int pm_s[kSmemPairs];   // 0 no term, 1 one 12-6 LJ term (pc_s), 2 general (pair_terms)
    __shared__ float qt_s[8];            // per-type charges (when charges are a function of type)
    const PairCoef* pc = nullptr;
    const int* pmode = nullptr;
    const float* qt = nullptr;
    if(MIXED && P.T * P.T <= kSmemPairs) {
        for(int q = threadIdx.x; q < P.T * P.T; q += blockDim.x) {
            PairCoef c{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            int mode = 0;
            const int cnt = d.nb_cnt[q];
            if(cnt == 1 && d.nb_kind[q * kMaxFF] == MTG_NB_LJ) {
                mode = 1;
                const float4 f = reinterpret_cast<const float4*>(d.nb_parf)[q * kMaxFF];
                c = PairCoef{f.x, f.y, f.z, f.w, P.lj_shift == 2 ? d.nb_fsf[q * kMaxFF] : 0.0f, 0.0f, 0.0f, 0.0f};
            } else if(cnt > 0) {
                mode = 2;
            }
            pc_s[q] = c;
            pm_s[q] = mode;
        }
        if(P.qtype && threadIdx.x < P.T) qt_s[threadIdx.x] = d.qtype[threadIdx.x];
        __syncthreads();
        pc = pc_s;
        pmode = pm_s;
        if(P.qtype) qt = qt_s;
    }
    const R gmax = R(262143.0) / ((R)P.rc + (R)P.rcoul + (R)P.skin);   // keeps |g d| < 2^18
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gt / TEAM, lane = gt % TEAM;
    const bool active = i < P.n;
    const bool mob = active && d.mobile[i] != 0;
    Fix fx{0, 0}, fy{0, 0}, fz{0, 0}, fu{0, 0};   // mixed: exact fixed point
    double bx = 0, by = 0, bz = 0, bu = 0;        // fp64
    if(mob) {
        const SysView v = sys_view(d, P, rep_of_atom(d, P, i));
        const R rc2 = (R)v.rc * (R)v.rc;
        const R rq2 = (R)v.rcoul * (R)v.rcoul;
        const R irc = R(1) / (R)v.rcoul;
        const float fs[3] = {v.fscale[0], v.fscale[1], v.fscale[2]};
        const uint4 qi4 = MIXED ? d.pq[i] : make_uint4(0, 0, 0, 0);
        const int ti = MIXED ? (int)qi4.w : d.type[i];
        const R qi = MIXED ? (R)d.qf[i] : (R)d.qd[i];
        const R kq = MIXED ? (R)kCoulombKf : (R)1389.32;
        const int cnt = min(d.vcount[i], d.vmax);   // an overflowed build is redone; stay in the row
        const uint32_t* lst = d.vlist + (size_t)i * d.vmax;
        int e = lane;
        for(; e + 3 * TEAM < cnt; e += 4 * TEAM) {
            uint32_t ent[4];
#pragma unroll
            for(int q = 0; q < 4; q++) ent[q] = __ldg(lst + e + q * TEAM);
#pragma unroll
            for(int q = 0; q < 4; q++) {
                R dx, dy, dz, g, u;
                pair_entry<MIXED, ENERGY, R>(d, P, i, ent[q], ti, qi, rc2, rq2, irc, kq, pc, pmode, qt, qi4, fs, dx, dy, dz, g, u);
                if(MIXED) {
                    g = fminf(fmaxf(g, -gmax), gmax);
                    fix_add(fx, (float)(g * dx));
                    fix_add(fy, (float)(g * dy));
                    fix_add(fz, (float)(g * dz));
                    if(ENERGY) fix_add_clamped(fu, (float)u);
                } else {
                    bx += (double)(g * dx); by += (double)(g * dy); bz += (double)(g * dz);
                    if(ENERGY) bu += (double)u;
                }
            }
        }
        for(; e < cnt; e += TEAM) {
            R dx, dy, dz, g, u;
            pair_entry<MIXED, ENERGY, R>(d, P, i, __ldg(lst + e), ti, qi, rc2, rq2, irc, kq, pc, pmode, qt, qi4, fs, dx, dy, dz, g, u);
            if(MIXED) {
                g = fminf(fmaxf(g, -gmax), gmax);
                fix_add(fx, (float)(g * dx));
                fix_add(fy, (float)(g * dy));
                fix_add(fz, (float)(g * dz));
                if(ENERGY) fix_add_clamped(fu, (float)u);
            } else {
                bx += (double)(g * dx); by += (double)(g * dy); bz += (double)(g * dz);
                if(ENERGY) bu += (double)u;
            }
        }
        // bonded terms of atom i, one entry per lane
        const int nbd = (d.bptr[i + 1] - d.bptr[i]) + (d.aptr[i + 1] - d.aptr[i]) + (d.dptr[i + 1] - d.dptr[i]);
        for(int b = lane; b < nbd; b += TEAM) {
            R gx = 0, gy = 0, gz = 0, gu = 0;
            bonded_entry<MIXED, R>(d, P, i, b, gx, gy, gz, gu, ENERGY);
            if(MIXED) {
                fix_add_clamped(fx, (float)gx);
                fix_add_clamped(fy, (float)gy);
                fix_add_clamped(fz, (float)gz);
                if(ENERGY) fix_add_clamped(fu, (float)gu);
            } else {
                bx += (double)gx; by += (double)gy; bz += (double)gz;
                if(ENERGY) bu += (double)gu;
            }
        }
    }
    // team reduction (integer: exact; FP64: fixed tree); teams are aligned within the warp
    if(MIXED) {
        long long ax = fix_total(fx), ay = fix_total(fy), az = fix_total(fz), au = ENERGY ? fix_total(fu) : 0;
        for(int o = TEAM / 2; o > 0; o >>= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, o);
            ay += __shfl_xor_sync(0xffffffffu, ay, o);
            az += __shfl_xor_sync(0xffffffffu, az, o);
            if(ENERGY) au += __shfl_xor_sync(0xffffffffu, au, o);
        }
        if(active && lane == 0) {
            d.Fx[i] = ax;
            d.Fy[i] = ay;
            d.Fz[i] = az;
            if(ENERGY) d.U[i] = double(au) * (1.0 / kFixScale);
        }
    } else {
        for(int o = TEAM / 2; o > 0; o >>= 1) {
            bx += __shfl_xor_sync(0xffffffffu, bx, o);
            by += __shfl_xor_sync(0xffffffffu, by, o);
            bz += __shfl_xor_sync(0xffffffffu, bz, o);
            if(ENERGY) bu += __shfl_xor_sync(0xffffffffu, bu, o);
        }
        if(active && lane == 0) {
            d.F[3 * i] = bx;
            d.F[3 * i + 1] = by;
            d.F[3 * i + 2] = bz;
            if(ENERGY) d.U[i] = bu;
        }
    }
}

// Conversions between the mixed-mode position/force formats and the FP64 host-facing arrays.
__global__ void k_sync_pos(DevSys d, Params P, int to_master) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n) return;
    if(to_master) {
        // d.r -> hi/lo (set_state)
        uint4 q = d.pq[i];
        q.w = (unsigned int)d.type[i];
        d.pq[i] = q;
        const SysView v = sys_view(d, P, rep_of_atom(d, P, i));
        store_pos(d, v.fconv, i, d.r[3 * i], d.r[3 * i + 1], d.r[3 * i + 2], true);
        float4 h = d.hi[i], l = d.lo[i];
        h.w = d.qf[i];
        l.w = __int_as_float(d.type[i]);
        d.hi[i] = h;
        d.lo[i] = l;
    } else {
        double x, y, z;
        load_pos(d, i, x, y, z, true);
        d.r[3 * i] = x;
        d.r[3 * i + 1] = y;
        d.r[3 * i + 2] = z;
    }
}

__global__ void k_forces_to_double(DevSys d, Params P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n) return;
    d.F[3 * i] = double(d.Fx[i]) * (1.0 / kFixScale);
    d.F[3 * i + 1] = double(d.Fy[i]) * (1.0 / kFixScale);
    d.F[3 * i + 2] = double(d.Fz[i]) * (1.0 / kFixScale);
}

__global__ void k_clear_rebuild(DevSys d) {
    if(threadIdx.x == 0 && blockIdx.x == 0 && d.sc->rebuild) {
        d.sc->rebuild = 0;
        d.sc->builds += 1;
    }
}

// Gradient-descent step of CSimulationBox::gradientDescentStep (SimulationBox.cpp:197-208):
// r += lr F, no clipping, no wrapping.  Also sums U, p^2/m and F.r (after the move) for the
// output line, and flags a production list rebuild when an atom moved beyond skin/2.
__global__ void k_gd_step(DevSys d, Params P, double lr, int mode) {
    __shared__ double smem[32 * 3];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    if(k < P.n) {
        const bool mixed = (mode == MTG_PREC_MIXED);
        double f[3], r[3];
        load_force(d, k, f[0], f[1], f[2], mixed);
        load_pos(d, k, r[0], r[1], r[2], mixed);
        double fr = 0.0, p2 = 0.0;
        for(int a = 0; a < 3; a++) {
            r[a] = r[a] + f[a] * lr;
            fr += f[a] * r[a];
            p2 += d.p[3 * k + a] * d.p[3 * k + a];
        }
        store_pos(d, P.fconv, k, r[0], r[1], r[2], mixed);
        if(mode != MTG_PREC_REFERENCE) {
            const double bx = minimg_d(r[0] - d.r_build[3 * k], P.box[0], 1.0 / P.box[0]);
            const double by = minimg_d(r[1] - d.r_build[3 * k + 1], P.box[1], 1.0 / P.box[1]);
            const double bz = minimg_d(r[2] - d.r_build[3 * k + 2], P.box[2], 1.0 / P.box[2]);
            const double h = 0.5 * double(P.skin);
            if(bx * bx + by * by + bz * bz > h * h) d.sc->rebuild = 1;
        }
        v[0] = d.U[k];
        v[1] = p2 / d.m[k];
        v[2] = fr;
    }
    block_sum<3>(v, smem);
    if(threadIdx.x == 0) {
        d.partial[blockIdx.x * 4 + 0] = v[0];
        d.partial[blockIdx.x * 4 + 1] = v[1];
        d.partial[blockIdx.x * 4 + 2] = v[2];
    }
    if(last_block(&d.sc->done_blocks)) {
        if(threadIdx.x == 0) {
            double sum[3] = {0.0, 0.0, 0.0};
            for(int b = 0; b < (int)gridDim.x; b++)
                for(int q = 0; q < 3; q++) sum[q] += d.partial[b * 4 + q];
            const double V = P.box[0] * P.box[1] * P.box[2];
            d.rec[0] = sum[0];
            d.rec[1] = 0.5 * sum[1];
            d.rec[2] = sum[1] / (3.0 * double(P.n));
            d.rec[3] = (1.0 / (3.0 * V)) * (sum[1] + sum[2]);
            d.rec[4] = V;
            d.sc->U = sum[0];
            d.sc->done_blocks = 0;
        }
    }
}

}  // namespace

static inline int nblk(int n, int t) { return (n + t - 1) / t; }

void launch_gd_step(const DevSys& d, const Params& P, double lr, cudaStream_t s) {
    k_gd_step<<<reduction_blocks(P.n), 256, 0, s>>>(d, P, lr, P.precision);
}

void launch_prologue(const DevSys& d, const Params& P, cudaStream_t s) {
    k_prologue<<<integration_blocks(P), 256, 0, s>>>(d, P);
}

void launch_prod_kick_drift(const DevSys& d, const Params& P, cudaStream_t s, cudaGraphConditionalHandle cond) {
    const int nb = integration_blocks(P);
    if(P.precision == MTG_PREC_MIXED) k_pkick_drift<true><<<nb, 256, 0, s>>>(d, P, cond);
    else k_pkick_drift<false><<<nb, 256, 0, s>>>(d, P, cond);
}

void launch_prod_build(const DevSys& d, const Params& P, bool force, cudaStream_t s) {
    const int ncell = P.nrep ? P.ncell_total : P.pnx * P.pny * P.pnz;
    if(force) cudaMemsetAsync(&d.sc->rebuild, 0xff, sizeof(int32_t), s);
    // counts are cleared unconditionally; the kernels below return early when no rebuild is due
    cudaMemsetAsync(d.pcell_count, 0, sizeof(int) * ncell, s);
    if(P.precision == MTG_PREC_MIXED) k_pcell_assign<true><<<nblk(P.n, 256), 256, 0, s>>>(d, P);
    else k_pcell_assign<false><<<nblk(P.n, 256), 256, 0, s>>>(d, P);
    k_pcell_scan<<<1, 1024, 0, s>>>(d, ncell);
    k_pcell_scatter<<<nblk(P.n, 256), 256, 0, s>>>(d, P);
    k_pcell_rank<<<nblk(ncell * 32, 256), 256, 0, s>>>(d, ncell);
    if(P.precision == MTG_PREC_MIXED) k_vlist<true><<<nblk(P.n * 32, 256), 256, 0, s>>>(d, P);
    else k_vlist<false><<<nblk(P.n * 32, 256), 256, 0, s>>>(d, P);
    k_clear_rebuild<<<1, 32, 0, s>>>(d);
}

template<bool MIXED, bool ENERGY>
static void force_team(const DevSys& d, const Params& P, cudaStream_t s) {
    const int team = P.team;
    const int nb = nblk(P.n * team, 256);
    if(team == 8) k_pforce<MIXED, ENERGY, 8><<<nb, 256, 0, s>>>(d, P);
    else if(team == 16) k_pforce<MIXED, ENERGY, 16><<<nb, 256, 0, s>>>(d, P);
    else k_pforce<MIXED, ENERGY, 32><<<nb, 256, 0, s>>>(d, P);
}

void launch_prod_force(const DevSys& d, const Params& P, bool energy, cudaStream_t s) {
    if(P.precision == MTG_PREC_MIXED) {
        if(energy) force_team<true, true>(d, P, s);
        else force_team<true, false>(d, P, s);
    } else {
        if(energy) force_team<false, true>(d, P, s);
        else force_team<false, false>(d, P, s);
    }
}

void launch_prod_kick2(const DevSys& d, const Params& P, bool output, cudaStream_t s) {
    const int nb = integration_blocks(P);
    if(P.precision == MTG_PREC_MIXED) {
        if(output) k_pkick2<true, true><<<nb, 256, 0, s>>>(d, P);
        else k_pkick2<true, false><<<nb, 256, 0, s>>>(d, P);
    } else {
        if(output) k_pkick2<false, true><<<nb, 256, 0, s>>>(d, P);
        else k_pkick2<false, false><<<nb, 256, 0, s>>>(d, P);
    }
}

void launch_prod_sync_positions(const DevSys& d, const Params& P, bool to_master, cudaStream_t s) {
    k_sync_pos<<<nblk(P.n, 256), 256, 0, s>>>(d, P, to_master ? 1 : 0);
}

void launch_prod_forces_to_double(const DevSys& d, const Params& P, cudaStream_t s) {
    k_forces_to_double<<<nblk(P.n, 256), 256, 0, s>>>(d, P);
}

}  // namespace mtg
