// Production kernels: analytic force field in FP64 or mixed precision, Verlet neighbour list with
// a skin, fused integrator kernels, and the reduction/thermostat prologue shared by all modes.
//
// Layout in HBM (per atom):
//   FP64 mode : r double[3] (master), p double[3], F double[3]
//   mixed     : hi float4 (x,y,z hi, charge), lo float4 (x,y,z lo, type bits) -- the positions
//               as double-float pairs -- pq uint4 (x,y,z as 32-bit box fractions, type) with a
//               copy pqs in cell order, ph / pl float4 (momenta as double-float pairs, 1/m in .w),
//               F int64 x3 (SoA, 2^26 units per kJ/mol/A); r and p double[3] are the masters the
//               host reads and writes (k_sync).
// Neighbour list: one row per slot (the atom's position in cell order at the last build) of
// uint32 entries, the partner's slot in the low 29 bits and the exclusion class of the pair (none,
// 1-2, 1-3, 1-4, same molecule; FunctorCalcForce.cpp:95-157) in the top 3 bits.  Pairs whose class
// scale is exactly 0 are left out of the list.  Rebuilt when an atom has moved more than skin/2
// since the last build.
//
// The force gather keeps the reference's structure (FunctorCalcForce.cpp:159-281): each atom sums
// its own bonded terms, its neighbours and (cutoff) Coulomb, using the full list, so no atomics are
// needed and the energy bookkeeping (pair energy once per pair, angle energy on the centre, half
// the dihedral energy on each centre atom) follows the reference.  Mixed mode rounds every pair
// contribution to int64 fixed point exactly, so a force does not depend on the summation order.
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

// Programmatic dependent launch: a step kernel captured with the programmatic-serialization
// attribute may be scheduled while its predecessor drains; it waits here until the predecessor
// has completed and its writes are visible, before reading anything, and at once allows its own
// successor to be scheduled.  Launched without the attribute both instructions return at once.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launches of the step kernels: with the programmatic-serialization attribute while a plain step
// graph is captured (set_pdl_launch), otherwise an ordinary launch.
bool g_pdl = false;

template<typename... KArgs, typename... Args>
void launch_step_kernel(void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, Args... args) {
    if(!g_pdl) {
        kern<<<grid, block, 0, s>>>(args...);
        return;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}


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
        if(P.ensemble == MTG_NPT && P.precision != MTG_PREC_REFERENCE) {
            // the box changes every step: the barostat state holds it and its derived fields
            const BaroDev* b = d.baro;
            v.cbase = 0; v.pnx = b->pn[0]; v.pny = b->pn[1]; v.pnz = b->pn[2];
            for(int a = 0; a < 3; a++) {
                v.box[a] = b->L[a];
                v.fconv[a] = b->conv[a];
                v.fscale[a] = b->fscale[a];
            }
        } else {
            v.cbase = 0; v.pnx = P.pnx; v.pny = P.pny; v.pnz = P.pnz;
            for(int a = 0; a < 3; a++) {
                v.box[a] = P.box[a];
                v.fconv[a] = P.fconv[a];
                v.fscale[a] = P.fscale[a];
            }
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

// List rebuilds.  StepScalars::rebuild of the system: 0 none due, -1 every list (a forced
// rebuild), 1 due somewhere; in a batch each replica's own flag then says whether its lists are
// rebuilt, so a replica rebuilds exactly when it would alone (its atoms moved half the skin).
__device__ __forceinline__ bool rebuild_due(const DevSys& d, const Params& P, int r) {
    const int g = d.sc->rebuild;
    if(g == 0) return false;
    if(g < 0 || !P.nrep || r < 0) return true;
    return d.rsc[r].rebuild != 0;
}
__device__ __forceinline__ void flag_rebuild(const DevSys& d, const Params& P, const SysView& v) {
    if(P.nrep) v.sc->rebuild = 1;
    if(d.sc->rebuild == 0) d.sc->rebuild = 1;   // a forced rebuild (-1) stays forced
}


// Totals of one system's block partials (blocks b0 .. b0+nb-1, four doubles each), summed by the
// whole last block: thread t adds blocks t, t + blockDim, ... in order, then the fixed shuffle
// tree of block_sum.  Deterministic; thread 0 receives the totals.  (The reference-precision
// kernels keep a single-thread sum in block order.)
template<int NV>
__device__ __forceinline__ void system_totals(const double* partial, int b0, int nb, double (&s)[NV], double* smem) {
#pragma unroll
    for(int q = 0; q < NV; q++) s[q] = 0.0;
    for(int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
        for(int q = 0; q < NV; q++) s[q] += partial[(size_t)(b0 + b) * 4 + q];
    block_sum<NV>(s, smem);
}

// Block sum of a double-float per thread: shuffle tree in double-float, then FP64 over the
// warps by thread 0 (the only thread that receives the result).
__device__ __forceinline__ double block_sum_df(DF v, double* smem) {
    for(int o = 16; o > 0; o >>= 1) {
        const DF w{__shfl_down_sync(0xffffffffu, v.h, o), __shfl_down_sync(0xffffffffu, v.l, o)};
        v = df_add(v, w);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if(lane == 0) smem[warp] = df_val(v);
    __syncthreads();
    double t = 0.0;
    if(threadIdx.x == 0)
        for(int w = 0; w < nw; w++) t += smem[w];
    __syncthreads();
    return t;
}

// ---------------------------------------------------------------------------------------------
// Prologue: sum p^2/m, then the first thermostat half-step of the coming step.
// ---------------------------------------------------------------------------------------------
template<bool DFLOAT>
__global__ void k_prologue(DevSys d, Params P) {
    __shared__ double smem[32 * 2];
    const SysView sv = sys_view(d, P, rep_of_block(d, P));
    const int k = sv.off + (blockIdx.x - sv.bbase) * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};   // sum p^2/m, sum F.r (NPT: G_eps of the first step, VelVerlet.cpp:60)
    if(k < sv.off + sv.n) {
        double px = d.p[3 * k], py = d.p[3 * k + 1], pz = d.p[3 * k + 2];
        if(P.precision == MTG_PREC_MIXED) {   // mixed: the double-float mirrors are current
            const float4 h = d.ph[k], l = d.pl[k];
            px = (double)h.x + (double)l.x;
            py = (double)h.y + (double)l.y;
            pz = (double)h.z + (double)l.z;
        }
        v[0] = (px * px + py * py + pz * pz) / d.m[k];
        if(P.ensemble == MTG_NPT)
            v[1] = P.precision == MTG_PREC_REFERENCE
                       ? d.F[3 * k] * d.r[3 * k] + d.F[3 * k + 1] * d.r[3 * k + 1] + d.F[3 * k + 2] * d.r[3 * k + 2]
                       : d.W[k];
    }
    block_sum<2>(v, smem);
    if(threadIdx.x == 0) {
        d.partial[blockIdx.x * 4] = v[0];
        d.partial[blockIdx.x * 4 + 1] = v[1];
    }
    if(last_block_of(&sv.sc->done_blocks, (unsigned)sv.nb)) {
        __shared__ double tot, tot_fr;
        double s2[2] = {0.0, 0.0};
        if(P.precision != MTG_PREC_REFERENCE) system_totals<2>(d.partial, sv.bbase, sv.nb, s2, smem);
        if(threadIdx.x == 0) {
            if(P.precision == MTG_PREC_REFERENCE) {
                for(int b = sv.bbase; b < sv.bbase + sv.nb; b++) {
                    s2[0] += d.partial[b * 4];
                    s2[1] += d.partial[b * 4 + 1];
                }
            }
            tot = s2[0];
            tot_fr = s2[1];
            sv.sc->done_blocks = 0;
        }
        __syncthreads();
        if(P.ensemble == MTG_NPT) {
            if(threadIdx.x < 96) npt_scalars<DFLOAT>(P, d, tot, 0.0, tot_fr, 0.0, false, false);
            if(threadIdx.x == 0) d.sc->c2 = 1.0;
            return;
        }
        if(threadIdx.x < 96) {
            double KE2 = tot;
            double c2 = 1.0, c1 = 1.0;
            Params Q = P;
            Q.n = sv.n;
            Q.kT = sv.kT;
            if(P.ensemble == MTG_NVT || P.ensemble == MTG_NPT)
                thermostat<DFLOAT>(Q, sv.sc, sv.th, sv.th_saved, KE2, false, &c2, &c1);
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

// Mixed mode also keeps each coordinate as a 32-bit fraction of the box, round(x / L * 2^32)
// modulo 2^32 (frac32_df).  The difference of two such coordinates, read as a signed 32-bit
// integer, is the minimum-image separation in units of L / 2^32, exact for any |dx| < L/2 (no
// cancellation at the periodic boundary).

__device__ __forceinline__ void store_pos(const DevSys& d, const double* conv, int i, double x, double y, double z,
                                          bool mixed) {
    if(mixed) {
        const DF X = df_of(x), Y = df_of(y), Z = df_of(z);
        float4 h = d.hi[i], l = d.lo[i];
        h.x = X.h; h.y = Y.h; h.z = Z.h;
        l.x = X.l; l.y = Y.l; l.z = Z.l;
        d.hi[i] = h;
        d.lo[i] = l;
        uint4 q = d.pq[i];
        q.x = frac32_df(X, df_of(conv[0]));
        q.y = frac32_df(Y, df_of(conv[1]));
        q.z = frac32_df(Z, df_of(conv[2]));
        d.pq[i] = q;
        d.pqs[d.slot_of[i]] = q;
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
__device__ __forceinline__ void kick_drift_atom(DevSys& d, const Params& P, const SysView& v, int k);

// FP64 mode.  One 256-atom block per launch block; a batch maps blocks to replicas (blk_rep).
__global__ void k_pkick_drift(DevSys d, Params P, cudaGraphConditionalHandle cond, int use_cond) {
    pdl_enter();
    const SysView v = sys_view(d, P, rep_of_block(d, P));
    const int k = v.off + (blockIdx.x - v.bbase) * blockDim.x + threadIdx.x;
    const bool mine = k < v.off + v.n;
    if(use_cond) {
        // inside a captured step graph: the last block hands the grid-wide rebuild decision to the
        // graph's IF node that wraps the list build
        if(mine) kick_drift_atom(d, P, v, k);
        if(last_block(&d.sc->done_blocks)) {
            if(threadIdx.x == 0) {
                d.sc->done_blocks = 0;
                cudaGraphSetConditional(cond, d.sc->rebuild ? 1u : 0u);
            }
        }
        return;
    }
    if(!mine) return;
    kick_drift_atom(d, P, v, k);
}

__device__ __forceinline__ void kick_drift_atom(DevSys& d, const Params& P, const SysView& v, int k) {
    const double S = v.sc->S;
    const bool npt = P.ensemble == MTG_NPT;
    double fx, fy, fz, x, y, z;
    load_force(d, k, fx, fy, fz, false);
    load_pos(d, k, x, y, z, false);
    double px, py, pz;
    double sb = 1.0, h2;
    if(npt) {
        // prop_p then prop_r with the coefficients of this step's barostat momentum
        // (VelVerlet.cpp:57-71, 124-150); the momenta carry the pending thermostat scale
        const BaroDev* b = d.baro;
        const double ap = b->ap, bp = b->bp, ar = b->ar, br = b->br;
        const double im = 1.0 / d.m[k];
        px = (d.p[3 * k] * S) * ap + fx * bp;
        py = (d.p[3 * k + 1] * S) * ap + fy * bp;
        pz = (d.p[3 * k + 2] * S) * ap + fz * bp;
        x = x * ar + (px * im) * br;
        y = y * ar + (py * im) * br;
        z = z * ar + (pz * im) * br;
        sb = (double)b->sb;
        h2 = (double)b->h2;
    } else {
        const double dt_2 = P.dt / 2.0;
        const double dm = P.dt / d.m[k];
        px = d.p[3 * k] * S + fx * dt_2;
        py = d.p[3 * k + 1] * S + fy * dt_2;
        pz = d.p[3 * k + 2] * S + fz * dt_2;
        x += px * dm;
        y += py * dm;
        z += pz * dm;
        const double h = 0.5 * double(v.skin);
        h2 = h * h;
    }
    d.p[3 * k] = px;
    d.p[3 * k + 1] = py;
    d.p[3 * k + 2] = pz;
    store_pos(d, v.fconv, k, x, y, z, false);
    // displacement since the last list build (minimum image: wrapping is not a displacement),
    // against the build positions scaled with the box under NPT; fconv 2^-32 = 1/L rounded,
    // without a division
    const double bx = minimg_d(x - d.r_build[3 * k] * sb, v.box[0], v.fconv[0] * 0x1p-32);
    const double by = minimg_d(y - d.r_build[3 * k + 1] * sb, v.box[1], v.fconv[1] * 0x1p-32);
    const double bz = minimg_d(z - d.r_build[3 * k + 2] * sb, v.box[2], v.fconv[2] * 0x1p-32);
    if(bx * bx + by * by + bz * bz > h2) flag_rebuild(d, P, v);
}

__device__ __forceinline__ double wrap_coord(double x, double Lm) {
    // pbcWrap (SimulationBox.cpp:135-166)
    const double h = Lm / 2.0;
    if(x >= h) x -= double((int)((x + h) / Lm)) * Lm;
    if(x < -h) x -= double((int)((x + (-h)) / Lm)) * Lm;
    return x;
}

// End-of-step scalar work of a system's last block (warps 0..2): thermostat and output record,
// with the replica's size, temperature and box for a batch.
template<bool DFLOAT>
__device__ __forceinline__ void step_end(const DevSys& d, const Params& P, const SysView& sv, const double* tot, bool output) {
    if(P.nrep) {
        Params Q = P;
        Q.n = sv.n;
        Q.kT = sv.kT;
        for(int a = 0; a < 3; a++) Q.box[a] = sv.box[a];
        end_of_step<DFLOAT>(Q, sv.sc, sv.th, sv.th_saved, tot[0], tot[2], tot[1], output, sv.rec);
        if(threadIdx.x == 0 && sv.sc->timeout) d.sc->timeout = 1;
        if(threadIdx.x == 0 && sv.sc->nonfinite) d.sc->nonfinite = 1;
    } else {
        end_of_step<DFLOAT>(P, d.sc, d.th, d.th_saved, tot[0], tot[2], tot[1], output, d.rec);
    }
}

// FP64 mode: second kick, clipping, pbcWrap, sums, end-of-step work.
template<bool OUTPUT>
__global__ void k_pkick2(DevSys d, Params P) {
    pdl_enter();
    __shared__ double smem[32 * 3];
    const SysView sv = sys_view(d, P, rep_of_block(d, P));
    const int k = sv.off + (blockIdx.x - sv.bbase) * blockDim.x + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    const bool npt = P.ensemble == MTG_NPT;
    if(k < sv.off + sv.n) {
        const double dt_2 = P.dt / 2.0;
        double f[3], r[3];
        load_force(d, k, f[0], f[1], f[2], false);
        load_pos(d, k, r[0], r[1], r[2], false);
        double p2 = 0.0, fr = 0.0;
        if(npt) {
            // 3.5 prop_p with the new forces (no clipping in the NPT branch, VelVerlet.cpp:57-71)
            const double ap = d.baro->ap, bp = d.baro->bp;
#pragma unroll
            for(int a = 0; a < 3; a++) {
                const double p = d.p[3 * k + a] * ap + f[a] * bp;
                d.p[3 * k + a] = p;
                r[a] = wrap_coord(r[a], sv.box[a]);
                p2 += p * p;
            }
        } else {
#pragma unroll
            for(int a = 0; a < 3; a++) {
                if(P.clip && P.fcut > 0.0 && fabs(f[a]) > P.fcut) {
                    f[a] = ((f[a] >= 0.0) ? 1.0 : -1.0) * P.fcut;
                    d.F[3 * k + a] = f[a];
                }
                const double p = d.p[3 * k + a] + f[a] * dt_2;
                d.p[3 * k + a] = p;
                r[a] = wrap_coord(r[a], sv.box[a]);
                p2 += p * p;
                fr += f[a] * r[a];
            }
        }
        store_pos(d, sv.fconv, k, r[0], r[1], r[2], false);
        v[0] = p2 / d.m[k];
        if(npt) v[1] = d.W[k];   // pair virial: every step drives the barostat
        else if(OUTPUT) v[1] = fr;
        if(OUTPUT) v[2] = d.U[k];
    }
    block_sum<3>(v, smem);
    if(threadIdx.x == 0) {
        d.partial[blockIdx.x * 4 + 0] = v[0];
        d.partial[blockIdx.x * 4 + 1] = v[1];
        d.partial[blockIdx.x * 4 + 2] = v[2];
    }
    if(last_block_of(&sv.sc->done_blocks, (unsigned)sv.nb)) {
        __shared__ double tot[3];
        double s3[3];
        system_totals<3>(d.partial, sv.bbase, sv.nb, s3, smem);
        if(threadIdx.x == 0) {
            for(int q = 0; q < 3; q++) tot[q] = s3[q];
            sv.sc->done_blocks = 0;
        }
        __syncthreads();
        if(threadIdx.x < 96) {
            if(npt) npt_scalars<false>(P, d, tot[0], tot[1], tot[1], tot[2], true, OUTPUT);
            else step_end<false>(d, P, sv, tot, OUTPUT);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Mixed-precision integration in double-float arithmetic (no FP64 instruction per atom).
// Per block, thread 0 turns the FP64 scalars into double-float constants.
// ---------------------------------------------------------------------------------------------
struct MixK {
    DF S, dt, dt2, fcut;
    DF conv[3], L[3];
    float Lf[3], iLf[3], L2f[3];
    float h2, fcutf;
    long long fcut_q;
};

__device__ __forceinline__ void mix_consts(const SysView& v, const Params& P, MixK& K) {
    K.S = df_of(v.sc->S);
    K.dt = df_of(P.dt);
    K.dt2 = df_of(P.dt / 2.0);
    for(int a = 0; a < 3; a++) {
        K.conv[a] = df_of(v.fconv[a]);
        K.L[a] = df_of(v.box[a]);
        K.Lf[a] = (float)v.box[a];
        K.iLf[a] = (float)(1.0 / v.box[a]);
        K.L2f[a] = (float)(0.5 * v.box[a]);
    }
    const float hs = 0.5f * v.skin;
    K.h2 = hs * hs;
    K.fcut = df_of(P.fcut);
    K.fcutf = (float)P.fcut;
    K.fcut_q = (long long)(P.fcut * kFixScale);
}

// The same from the constants converted once on the host (MixConst): only the pending scale S
// changes from step to step.
__device__ __forceinline__ void mix_load(const DevSys& d, const SysView& v, int rep, MixK& K) {
    const MixConst& m = d.mixk[rep < 0 ? 0 : rep];
    K.S = df_of(v.sc->S);
    K.dt = m.dt;
    K.dt2 = m.dt2;
    for(int a = 0; a < 3; a++) {
        K.conv[a] = m.conv[a];
        K.L[a] = m.L[a];
        K.Lf[a] = m.Lf[a];
        K.iLf[a] = m.iLf[a];
        K.L2f[a] = m.L2f[a];
    }
    K.h2 = m.h2;
    K.fcut = m.fcut;
    K.fcutf = m.fcutf;
    K.fcut_q = m.fcut_q;
}

// p <- S p + dt/2 F, r <- r + dt p / m (VelVerlet.cpp:74-93 with the pending thermostat scale),
// box fractions, and the half-skin displacement test against the positions of the last list build.
__global__ void k_mkick_drift(DevSys d, Params P, cudaGraphConditionalHandle cond, int use_cond) {
    pdl_enter();
    __shared__ MixK K;
    const int rep = rep_of_block(d, P);
    const SysView v = sys_view(d, P, rep);
    // the atom's loads are issued before the block waits for the constants
    const int k = v.off + (blockIdx.x - v.bbase) * blockDim.x + threadIdx.x;
    const bool mine = k < v.off + v.n;
    float4 h, l, ph, pl, rb;
    long long fq[3];
    int slot = 0;
    if(mine) {
        h = d.hi[k];
        l = d.lo[k];
        ph = d.ph[k];
        pl = d.pl[k];
        rb = d.rb4[k];
        fq[0] = d.Fx[k];
        fq[1] = d.Fy[k];
        fq[2] = d.Fz[k];
        slot = d.slot_of[k];
    }
    if(threadIdx.x == 0) mix_load(d, v, rep, K);
    __syncthreads();
    if(mine) {
        const DF dtm = df_mul(K.dt, DF{ph.w, pl.w});
        DF p[3] = {{ph.x, pl.x}, {ph.y, pl.y}, {ph.z, pl.z}};
        DF x[3] = {{h.x, l.x}, {h.y, l.y}, {h.z, l.z}};
        const float rbv[3] = {rb.x, rb.y, rb.z};
        unsigned int q[3];
        float d2 = 0.0f;
#pragma unroll
        for(int a = 0; a < 3; a++) {
            p[a] = df_add(df_mul(p[a], K.S), df_mul(df_fix(fq[a]), K.dt2));
            x[a] = df_add(x[a], df_mul(p[a], dtm));
            q[a] = frac32_df(x[a], K.conv[a]);
            const float dd = minimg_f(__fsub_rn(x[a].h, rbv[a]) + x[a].l, K.Lf[a], K.iLf[a]);
            d2 += dd * dd;
        }
        d.ph[k] = make_float4(p[0].h, p[1].h, p[2].h, ph.w);
        d.pl[k] = make_float4(p[0].l, p[1].l, p[2].l, pl.w);
        d.hi[k] = make_float4(x[0].h, x[1].h, x[2].h, h.w);
        d.lo[k] = make_float4(x[0].l, x[1].l, x[2].l, l.w);
        const uint4 qk = make_uint4(q[0], q[1], q[2], (unsigned int)__float_as_int(l.w));
        d.pq[k] = qk;
        d.pqs[slot] = qk;   // the force gather reads positions in cell (slot) order
        if(d2 > K.h2) flag_rebuild(d, P, v);
    }
    if(use_cond) {
        // inside a captured step graph: the last block hands the grid-wide rebuild decision to the
        // graph's IF node that wraps the list build
        if(last_block(&d.sc->done_blocks)) {
            if(threadIdx.x == 0) {
                d.sc->done_blocks = 0;
                cudaGraphSetConditional(cond, d.sc->rebuild ? 1u : 0u);
            }
        }
    }
}

// NPT, mixed mode: 3.2 prop_p and 3.3 prop_r (VelVerlet.cpp:57-71, 124-150) in double-float with
// the coefficients of this step's barostat momentum (the momenta carry the pending thermostat
// scale), box fractions in this step's box, and the displacement test against the build positions
// scaled with the box (baro_box_fields).
__global__ void k_mkick_drift_npt(DevSys d, Params P, cudaGraphConditionalHandle cond, int use_cond) {
    pdl_enter();
    __shared__ MixK K;
    __shared__ DF ap, bp, ar, br;
    __shared__ float sb, h2;
    const SysView v = sys_view(d, P, -1);
    if(threadIdx.x == 0) {
        mix_consts(v, P, K);
        const BaroDev* b = d.baro;
        ap = df_of(b->ap);
        bp = df_of(b->bp);
        ar = df_of(b->ar);
        br = df_of(b->br);
        sb = b->sb;
        h2 = b->h2;
    }
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k < P.n) {
        const float4 h = d.hi[k], l = d.lo[k], ph = d.ph[k], pl = d.pl[k], rb = d.rb4[k];
        const DF im{ph.w, pl.w};
        const long long fq[3] = {d.Fx[k], d.Fy[k], d.Fz[k]};
        DF p[3] = {{ph.x, pl.x}, {ph.y, pl.y}, {ph.z, pl.z}};
        DF x[3] = {{h.x, l.x}, {h.y, l.y}, {h.z, l.z}};
        const float rbv[3] = {rb.x, rb.y, rb.z};
        unsigned int q[3];
        float d2 = 0.0f;
#pragma unroll
        for(int a = 0; a < 3; a++) {
            p[a] = df_add(df_mul(df_mul(p[a], K.S), ap), df_mul(df_fix(fq[a]), bp));
            x[a] = df_add(df_mul(x[a], ar), df_mul(df_mul(p[a], im), br));
            q[a] = frac32_df(x[a], K.conv[a]);
            const float dd = minimg_f(__fsub_rn(x[a].h, __fmul_rn(rbv[a], sb)) + x[a].l, K.Lf[a], K.iLf[a]);
            d2 += dd * dd;
        }
        d.ph[k] = make_float4(p[0].h, p[1].h, p[2].h, ph.w);
        d.pl[k] = make_float4(p[0].l, p[1].l, p[2].l, pl.w);
        d.hi[k] = make_float4(x[0].h, x[1].h, x[2].h, h.w);
        d.lo[k] = make_float4(x[0].l, x[1].l, x[2].l, l.w);
        const uint4 qk = make_uint4(q[0], q[1], q[2], (unsigned int)__float_as_int(l.w));
        d.pq[k] = qk;
        d.pqs[d.slot_of[k]] = qk;
        if(d2 > h2) flag_rebuild(d, P, v);
    }
    if(use_cond) {
        if(last_block(&d.sc->done_blocks)) {
            if(threadIdx.x == 0) {
                d.sc->done_blocks = 0;
                cudaGraphSetConditional(cond, d.sc->rebuild ? 1u : 0u);
            }
        }
    }
}

// NPT, mixed mode: 3.5 prop_p with the new forces (no clipping in the NPT branch), wrap into the
// current box, block sums of p^2/m, of the pair virial and (output steps) of U.
template<bool OUTPUT>
__global__ void k_mkick2_npt(DevSys d, Params P) {
    pdl_enter();
    __shared__ MixK K;
    __shared__ DF ap, bp;
    __shared__ double smem[32 * 3];
    const SysView sv = sys_view(d, P, -1);
    if(threadIdx.x == 0) {
        mix_consts(sv, P, K);
        ap = df_of(d.baro->ap);
        bp = df_of(d.baro->bp);
    }
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    DF ke{0.0f, 0.0f};
    double v[3] = {0.0, 0.0, 0.0};
    if(k < P.n) {
        float4 h = d.hi[k], l = d.lo[k];
        const float4 ph = d.ph[k], pl = d.pl[k];
        const long long fq[3] = {d.Fx[k], d.Fy[k], d.Fz[k]};
        DF p[3] = {{ph.x, pl.x}, {ph.y, pl.y}, {ph.z, pl.z}};
        DF x[3] = {{h.x, l.x}, {h.y, l.y}, {h.z, l.z}};
        DF p2{0.0f, 0.0f};
        bool wrapped = false;
#pragma unroll
        for(int a = 0; a < 3; a++) {
            p[a] = df_add(df_mul(p[a], ap), df_mul(df_fix(fq[a]), bp));
            if(x[a].h >= K.L2f[a] || x[a].h < -K.L2f[a]) {
                const float m = floorf(__fmul_rn(__fadd_rn(x[a].h, K.L2f[a]), K.iLf[a]));
                x[a] = df_add(x[a], df_mul_f(K.L[a], -m));
                wrapped = true;
            }
            p2 = df_add(p2, df_mul(p[a], p[a]));
        }
        d.ph[k] = make_float4(p[0].h, p[1].h, p[2].h, ph.w);
        d.pl[k] = make_float4(p[0].l, p[1].l, p[2].l, pl.w);
        if(wrapped) {
            d.hi[k] = make_float4(x[0].h, x[1].h, x[2].h, h.w);
            d.lo[k] = make_float4(x[0].l, x[1].l, x[2].l, l.w);
        }
        ke = df_mul(p2, DF{ph.w, pl.w});
        v[1] = d.W[k];
        if(OUTPUT) v[2] = d.U[k];
    }
    const double ke_blk = block_sum_df(ke, smem);
    block_sum<3>(v, smem);
    if(threadIdx.x == 0) {
        d.partial[blockIdx.x * 4 + 0] = ke_blk;
        d.partial[blockIdx.x * 4 + 1] = v[1];
        d.partial[blockIdx.x * 4 + 2] = v[2];
    }
}

// Second kick with force clipping (VelVerlet.cpp:87,96-122), wrap into [-L/2, L/2) (the box
// fractions are periodic and stay as they are), block sums of p^2/m (and on output steps F.r and
// U).  The end-of-step scalar work runs in k_mstep_end: kept out of this kernel, the double-float
// chain's registers do not limit the occupancy of the per-atom pass.
template<bool OUTPUT>
__global__ void k_mkick2(DevSys d, Params P) {
    pdl_enter();
    __shared__ MixK K;
    __shared__ double smem[32 * 3];
    const int rep = rep_of_block(d, P);
    const SysView sv = sys_view(d, P, rep);
    // the atom's loads are issued before the block waits for the constants
    const int k = sv.off + (blockIdx.x - sv.bbase) * blockDim.x + threadIdx.x;
    const bool mine = k < sv.off + sv.n;
    float4 h, l, ph, pl;
    long long fq[3];
    double uk = 0.0;
    if(mine) {
        h = d.hi[k];
        l = d.lo[k];
        ph = d.ph[k];
        pl = d.pl[k];
        fq[0] = d.Fx[k];
        fq[1] = d.Fy[k];
        fq[2] = d.Fz[k];
        if(OUTPUT) uk = d.U[k];
    }
    if(threadIdx.x == 0) mix_load(d, sv, rep, K);
    __syncthreads();
    DF ke{0.0f, 0.0f};
    double v[3] = {0.0, 0.0, 0.0};
    if(mine) {
        DF p[3] = {{ph.x, pl.x}, {ph.y, pl.y}, {ph.z, pl.z}};
        DF x[3] = {{h.x, l.x}, {h.y, l.y}, {h.z, l.z}};
        DF p2{0.0f, 0.0f};
        bool wrapped = false;
        double fr = 0.0;
#pragma unroll
        for(int a = 0; a < 3; a++) {
            DF f = df_fix(fq[a]);
            if(P.clip && P.fcut > 0.0 && fabsf(f.h) > K.fcutf) {
                const bool pos = f.h >= 0.0f;
                f = pos ? K.fcut : df_neg(K.fcut);
                const long long c = pos ? K.fcut_q : -K.fcut_q;
                if(a == 0) d.Fx[k] = c; else if(a == 1) d.Fy[k] = c; else d.Fz[k] = c;
            }
            p[a] = df_add(p[a], df_mul(f, K.dt2));
            if(x[a].h >= K.L2f[a] || x[a].h < -K.L2f[a]) {
                const float m = floorf(__fmul_rn(__fadd_rn(x[a].h, K.L2f[a]), K.iLf[a]));
                x[a] = df_add(x[a], df_mul_f(K.L[a], -m));
                wrapped = true;
            }
            p2 = df_add(p2, df_mul(p[a], p[a]));
            if(OUTPUT) fr += df_val(f) * df_val(x[a]);
        }
        d.ph[k] = make_float4(p[0].h, p[1].h, p[2].h, ph.w);
        d.pl[k] = make_float4(p[0].l, p[1].l, p[2].l, pl.w);
        if(wrapped) {
            d.hi[k] = make_float4(x[0].h, x[1].h, x[2].h, h.w);
            d.lo[k] = make_float4(x[0].l, x[1].l, x[2].l, l.w);
        }
        ke = df_mul(p2, DF{ph.w, pl.w});
        if(OUTPUT) {
            v[1] = fr;
            v[2] = uk;
        }
    }
    const double ke_blk = block_sum_df(ke, smem);
    if(OUTPUT) block_sum<3>(v, smem);
    if(threadIdx.x == 0) {
        d.partial[blockIdx.x * 4 + 0] = ke_blk;
        d.partial[blockIdx.x * 4 + 1] = v[1];
        d.partial[blockIdx.x * 4 + 2] = v[2];
    }
}

// End of a mixed-precision step, one 96-thread block per system (per replica of a batch): the
// system's totals from its block partials, then the thermostat half-steps and the output record.
template<bool OUTPUT>
__global__ void __launch_bounds__(96, 1) k_mstep_end(DevSys d, Params P) {
    pdl_enter();
    __shared__ double smem[32 * 3];
    __shared__ double tot[3];
    const SysView sv = sys_view(d, P, P.nrep ? (int)blockIdx.x : -1);
    constexpr int NV = OUTPUT ? 3 : 1;   // F.r and U only on output steps
    double sv3[NV];
    system_totals<NV>(d.partial, sv.bbase, sv.nb, sv3, smem);
    if(threadIdx.x == 0) {
        tot[0] = sv3[0];
        tot[1] = OUTPUT ? sv3[NV > 1 ? 1 : 0] : 0.0;
        tot[2] = OUTPUT ? sv3[NV > 2 ? 2 : 0] : 0.0;
    }
    __syncthreads();
    step_end<true>(d, P, sv, tot, OUTPUT);
}

// NPT, mixed mode: the system's totals (the pair virial drives the barostat every step), then the
// barostat and chain half-steps, the output record and the next step's box (npt_scalars).
template<bool OUTPUT>
__global__ void __launch_bounds__(96, 1) k_mstep_end_npt(DevSys d, Params P) {
    pdl_enter();
    __shared__ double smem[32 * 3];
    __shared__ double tot[3];
    const SysView sv = sys_view(d, P, -1);
    double s3[3];
    system_totals<3>(d.partial, sv.bbase, sv.nb, s3, smem);
    if(threadIdx.x == 0)
        for(int q = 0; q < 3; q++) tot[q] = s3[q];
    __syncthreads();
    npt_scalars<true>(P, d, tot[0], tot[1], tot[1], tot[2], true, OUTPUT);
}

// ---------------------------------------------------------------------------------------------
// Verlet list build: cell grid with edge >= rlist (or one cell for small boxes), counting sort
// with a per-cell rank pass (deterministic order), then one warp per atom scanning the 27 cells.
// ---------------------------------------------------------------------------------------------
template<bool MIXED>
__global__ void k_pcell_assign(DevSys d, Params P) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n || !rebuild_due(d, P, rep_of_atom(d, P, i))) return;
    if(P.ensemble == MTG_NPT && i == 0) {
        // the list is built in the current box: displacements count from here (the box fields
        // the rest of this build reads do not change)
        BaroDev* b = d.baro;
        for(int a = 0; a < 3; a++) b->Lb[a] = b->L[a];
        const float hs = 0.5f * P.skin;
        b->sb = 1.0f;
        b->h2 = hs * hs;
    }
    double x, y, z;
    load_pos(d, i, x, y, z, MIXED);
    d.r_build[3 * i] = x;
    d.r_build[3 * i + 1] = y;
    d.r_build[3 * i + 2] = z;
    d.rb4[i] = make_float4((float)x, (float)y, (float)z, __int_as_float(d.type[i]));
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

// Exclusive scan of one system's cell counts (one block per replica of a batch): the replica's
// cells map onto its own slot range, so replicas rebuild independently.
__global__ void k_pcell_scan(DevSys d, Params P) {
    pdl_enter();
    const int r = P.nrep ? (int)blockIdx.x : -1;
    if(!rebuild_due(d, P, r)) return;
    const SysView v = sys_view(d, P, r);   // cell counts of the current box (NPT: of this build)
    const int cbase = v.cbase;
    const int ncell = v.pnx * v.pny * v.pnz;
    const int slot0 = P.nrep ? d.reps[r].off : 0;
    __shared__ int warp_tot[32];
    __shared__ int carry;
    if(threadIdx.x == 0) carry = slot0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for(int base = 0; base < ncell; base += blockDim.x) {
        const int c = base + threadIdx.x;
        const int v = (c < ncell) ? d.pcell_count[cbase + c] : 0;
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
            d.pcell_first[cbase + c] = excl;
            d.pcell_cursor[cbase + c] = 0;
        }
        __syncthreads();
        if(threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
}

__global__ void k_pcell_scatter(DevSys d, Params P) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n || !rebuild_due(d, P, rep_of_atom(d, P, i))) return;
    const int c = d.pcell_of[i];
    const int slot = atomicAdd(&d.pcell_cursor[c], 1);
    // vcount doubles as scratch until the list kernel: the atom's sort key, its type above its
    // index (index alone with more than 8 types)
    d.vcount[d.pcell_first[c] + slot] = (int)(P.T <= 8 ? ((unsigned)d.type[i] << kClassShift) | (unsigned)i : (unsigned)i);
}

// Atoms of a cell ordered by type and index (a rank pass, deterministic).  The position in the
// resulting cell order is the atom's slot: the Verlet list is kept per slot with partners named by
// slot, and the positions the force gather reads are copied into slot order, so the partners of
// the atoms a block works on lie in a compact, cache-resident range.
__global__ void k_pcell_rank(DevSys d, Params P, bool mixed) {
    pdl_enter();
    // one thread per position of the scratch array (positions are grouped by cell; a replica's
    // positions are its own atom range): the rank of its key among its cell's keys is its slot
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t >= P.n || !rebuild_due(d, P, rep_of_atom(d, P, t))) return;
    const unsigned* tmp = reinterpret_cast<const unsigned*>(d.vcount);
    // order within the cell: by type, then by index (the keys k_pcell_scatter wrote;
    // deterministic); atoms of one type sit together, so the atoms a warp's force gather takes
    // have alike rows (same split into short-range and Coulomb-only pairs, similar lengths)
    const unsigned kv = tmp[t];
    const int v = (int)(kv & kIdxMask);
    const int c = d.pcell_of[v];
    const int cnt = d.pcell_count[c], first = d.pcell_first[c];
    int rank = 0;
    for(int b = 0; b < cnt; b++) rank += (tmp[first + b] < kv);
    const int slot = first + rank;
    d.pcell_list[slot] = v;
    d.slot_of[v] = slot;
    d.rb4s[slot] = d.rb4[v];
    if(mixed) d.pqs[slot] = d.pq[v];
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
    pdl_enter();
    if(!d.sc->rebuild) return;
    const int si = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if(si >= P.n) return;
    const int i = d.pcell_list[si];
    if(!rebuild_due(d, P, rep_of_atom(d, P, i))) return;
    const SysView v = sys_view(d, P, rep_of_atom(d, P, i));
    const float rfull = fmaxf(v.rc, P.coulomb != MTG_COULOMB_ALLPAIRS ? v.rcoul : 0.0f);
    // FP32 distances: rounding (~1e-6 A) is far inside the skin margin
    const float4 ri = d.rb4s[si];
    const int ti = __float_as_int(ri.w);
    // list radius of pair (ti, tj): its own short-range cutoff (at most rc), widened to rcoul when
    // charges are on, plus the skin; a pair outside that radius cannot interact before the next
    // rebuild, which comes once any atom has moved half the skin
    const float rq = P.qon ? v.rcoul : 0.0f;
    auto list_r2 = [&](int tj) -> float {
        const float c = d.pair_cut[ti * P.T + tj];
        const float r = (c < 0.0f) ? rfull : fmaxf(fminf(c, v.rc), rq);
        return r > 0.0f ? (r + v.skin) * (r + v.skin) : -1.0f;
    };
    const float Lx = (float)v.box[0], Ly = (float)v.box[1], Lz = (float)v.box[2];
    const float iLx = 1.0f / Lx, iLy = 1.0f / Ly, iLz = 1.0f / Lz;
    const int ci = d.pcell_of[i] - v.cbase;
    const int cx = ci % v.pnx, cy = (ci / v.pnx) % v.pny, cz = ci / (v.pnx * v.pny);
    const int sx = v.pnx >= 3 ? 3 : 1, sy = v.pny >= 3 ? 3 : 1, sz = v.pnz >= 3 ? 3 : 1;
    // pairs with short-range terms fill the row from the front, Coulomb-only pairs from the back;
    // the back segment then moves behind the front one, so the force gather runs the short-range
    // arithmetic only where it applies
    uint32_t* out = d.vlist + (size_t)si * d.vmax;
    int cnt = 0, cq = 0;
    const int* nbc = d.nb_cnt + ti * P.T;
    for(int oz = 0; oz < sz; oz++) {
        const int z = sz == 1 ? 0 : (cz + oz - 1 + v.pnz) % v.pnz;
        for(int oy = 0; oy < sy; oy++) {
            const int y = sy == 1 ? 0 : (cy + oy - 1 + v.pny) % v.pny;
            for(int ox = 0; ox < sx; ox++) {
                const int x = sx == 1 ? 0 : (cx + ox - 1 + v.pnx) % v.pnx;
                const int c = v.cbase + x + v.pnx * (y + v.pny * z);
                const int first = d.pcell_first[c], n = d.pcell_count[c];
                for(int base = 0; base < n; base += 32) {
                    bool take = false, sr = false;
                    uint32_t entry = 0;
                    if(base + lane < n) {
                        const int sj = first + base + lane;
                        if(sj != si) {
                            const float4 rj = d.rb4s[sj];
                            const float dx = minimg_f(ri.x - rj.x, Lx, iLx);
                            const float dy = minimg_f(ri.y - rj.y, Ly, iLy);
                            const float dz = minimg_f(ri.z - rj.z, Lz, iLz);
                            const int tj = __float_as_int(rj.w);
                            if(dx * dx + dy * dy + dz * dz < list_r2(tj)) {
                                const int cls = excl_class(d, i, d.pcell_list[sj]);
                                if(P.scale[cls] != 0.0f) {
                                    take = true;
                                    sr = nbc[tj] > 0;
                                    entry = (uint32_t)sj | ((uint32_t)cls << kClassShift);
                                }
                            }
                        }
                    }
                    const unsigned below = (1u << lane) - 1u;
                    const unsigned bsr = __ballot_sync(0xffffffffu, take && sr);
                    const unsigned bq = __ballot_sync(0xffffffffu, take && !sr);
                    if(take && sr) {
                        const int slot = cnt + __popc(bsr & below);
                        if(slot < d.vmax) out[slot] = entry;
                    } else if(take) {
                        const int slot = d.vmax - 1 - (cq + __popc(bq & below));
                        if(slot >= 0) out[slot] = entry;
                    }
                    cnt += __popc(bsr);
                    cq += __popc(bq);
                }
            }
        }
    }
    const int total = cnt + cq;
    if(total <= d.vmax) {
        // move the Coulomb-only entries [vmax - cq, vmax) to [cnt, cnt + cq): the destination lies
        // below the source, so copying upwards in warp-wide chunks (each read before it is
        // written) never reads an overwritten entry
        for(int b = 0; b < cq; b += 32) {
            uint32_t v = 0;
            if(b + lane < cq) v = out[d.vmax - cq + b + lane];
            __syncwarp();
            if(b + lane < cq) out[cnt + b + lane] = v;
            __syncwarp();
        }
    }
    if(lane == 0) {
        d.vcount[si] = total;
        d.vsr[si] = cnt;
        if(total > d.vmax) {
            d.sc->overflow = 1;
            atomicMax(&d.sc->needed, total);
        }
    }
}

// ---------------------------------------------------------------------------------------------
// Force gather
// ---------------------------------------------------------------------------------------------
// Fixed-point accumulation of FP32 contributions (mixed mode) without the FP64 unit (which also
// executes 64-bit conversions, at a small fraction of the FP32 rate on this GPU).
// A contribution f becomes round(f * 2^26) exactly, split over two int32 accumulators.  With
// x = 16 f (|x| < 2^22) and M = 1.5 * 2^23:
//   tx = x + M          rounds x to the integer grid (the sum lies in [2^23, 2^24), ulp 1)
//   rx = x + (M - tx)   the remainder x - round(x), exact (|rx| <= 1/2)
//   ty = rx * 2^22 + M  (one fused operation; the product is exact) rounds it to the 2^-22 grid
//   h += bits(tx) - bits(M) = round(x),   l += bits(ty) - bits(M)
// and the lane's total is h * 2^22 + l in units of 2^-26 kJ/(mol A).  Every step is exact in FP32,
// so the fixed-point value of each contribution, and hence every sum of them, is independent of
// the order of summation and of zero contributions.  Callers pass x = 16 f with |f| clamped to
// 2^18 (no physical pair force comes near it); the scale 16 folds into the force factor.
struct Fix {
    int h, l;
};
__device__ __forceinline__ void fix_add16(Fix& a, float x) {
    const float M = 12582912.0f;
    const float tx = __fadd_rn(x, M);
    const float rx = __fadd_rn(x, __fsub_rn(M, tx));
    a.h += __float_as_int(tx) - __float_as_int(M);
    const float ty = __fmaf_rn(rx, 4194304.0f, M);
    a.l += __float_as_int(ty) - __float_as_int(M);
}
__device__ __forceinline__ void fix_add_clamped(Fix& a, float f) {
    fix_add16(a, __fmul_rn(fminf(fmaxf(f, -262143.0f), 262143.0f), 16.0f));
}
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
// With `energy` it also adds atom k's share of the term's virial, (r_k - r_X) . F_k with X a
// fixed atom of the term (a bond's or a dihedral's lowest-index atom, an angle's centre): summed
// over the term's atoms this is the term's virial sum_a r_a . F_a, because its forces sum to
// zero.  The relative vectors are the minimum-image ones the force uses.
template<bool MIXED, class R>
__device__ void bonded_entry(const DevSys& d, const Params& P, int k, int e, R& fx, R& fy, R& fz, R& u, R& w,
                             bool energy) {
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
        if(energy && k > i) w += s * (dx * dx + dy * dy + dz * dz);   // (r_k - r_i) . F_k
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
            if(energy) w -= dU * (ux * g1x + uy * g1y + uz * g1z);   // (r_k - r_centre) . F_k
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
        const R Fx = -dV * sgn * gx, Fy = -dV * sgn * gy, Fz = -dV * sgn * gz;
        fx += Fx; fy += Fy; fz += Fz;
        if(energy) {
            // r_k - r_X along the chain a-b-c-dd (k is a, or b for a centre entry), X the
            // lowest-index atom of the four
            int X = a;
            if(b < X) X = b;
            if(c < X) X = c;
            if(dd < X) X = dd;
            const bool kb = d.dcen[q] != 0;
            R rx = 0, ry = 0, rz = 0;                       // r_k - r_X
            if(X == a) {
                if(kb) { rx = b1x; ry = b1y; rz = b1z; }
            } else if(X == b) {
                if(!kb) { rx = -b1x; ry = -b1y; rz = -b1z; }
            } else if(X == c) {
                rx = -b2x; ry = -b2y; rz = -b2z;
                if(!kb) { rx -= b1x; ry -= b1y; rz -= b1z; }
            } else {
                rx = -b2x - b3x; ry = -b2y - b3y; rz = -b2z - b3z;
                if(!kb) { rx -= b1x; ry -= b1y; rz -= b1z; }
            }
            w += rx * Fx + ry * Fy + rz * Fz;
        }
    }
}

// One neighbour-list entry of atom i (FP64 path): force factor g (F_i += g * d) and pair energy u.
template<bool ENERGY>
// ri: atom i's position; L, iL: the box and its inverse (row constants, so that no FP64 division
// runs per pair).
__device__ __forceinline__ void pair_entry_d(const DevSys& d, const Params& P, int i, uint32_t ent, int ti, double qi,
                                             double rc2, double rq2, double irc, const double (&ri)[3],
                                             const double (&L)[3], const double (&iL)[3], double& dx, double& dy,
                                             double& dz, double& g, double& u) {
    const int j = (int)(ent & kIdxMask);
    const int cls = (int)(ent >> kClassShift);
    dx = minimg_d(ri[0] - d.r[3 * j], L[0], iL[0]);
    dy = minimg_d(ri[1] - d.r[3 * j + 1], L[1], iL[1]);
    dz = minimg_d(ri[2] - d.r[3 * j + 2], L[2], iL[2]);
    const int tj = d.type[j];
    const double r2 = dx * dx + dy * dy + dz * dz;
    const double ir = rsqrt(r2);   // within an ulp of 1/sqrt, without the FP64 division
    const double ir2 = ir * ir;
    g = 0;
    u = 0;
    if(r2 < rc2 && r2 >= 1e-6) pair_terms<double>(d, ti * P.T + tj, r2, ir, ir2, g, u, ENERGY, P.lj_shift);
    if(P.qon && r2 < rq2) {
        const double qq = 1389.32 * qi * d.qd[j];
        if(P.coulomb == MTG_COULOMB_SHIFTED) {
            g += qq * (ir2 - irc * irc) * ir;
            if(ENERGY) u += qq * (ir - irc + (r2 * ir - 1.0 / irc) * irc * irc);
        } else {
            g += qq * ir2 * ir;
            if(ENERGY) u += qq * ir;
        }
    }
    if(cls) {
        const double sc = (double)P.scale[cls];
        g *= sc;
        u *= sc;
    }
    if(!(ENERGY && j > i)) u = 0;
}

// Per type pair, staged in shared memory by the mixed force kernel: a single 12-6 LJ term
// (a, b, fs) with own2 = its squared own cutoff (FLT_MAX: the global cutoff only); own2 = 0 for a
// pair without short-range terms (the LJ arithmetic then runs on zero coefficients and is
// discarded, which costs less than a divergent branch); own2 < 0 for anything else (evaluated by
// pair_terms from global memory).
struct PairCoef {
    float a, b;       // 4 eps sigma^12, 4 eps alpha sigma^6
    float own2;       // see above
    float fs;         // force at the cutoff (force-shifted LJ), else 0
};
constexpr int kSmemPairs = 64;   // type pairs staged (T <= 8)

// One list entry of the atom in slot si in FP32 (mixed path), added to the fixed-point sums
// (fx, fy, fz, fu): every contribution is rounded to the 2^-26 grid exactly and summed as an
// integer, so a force depends neither on the order of the list nor on out-of-range entries nor on
// how its row is split over lanes.  The cutoff tests select instead of branching: out-of-range
// entries, about a quarter of a list with a skin, would otherwise split the warp.  g is clamped
// to gmax so that |g d| < 2^18.
// SR = false: a pair without short-range terms (the row's Coulomb-only segment), Coulomb alone.
template<bool ENERGY, bool SR>
__device__ __forceinline__ void pair_mixed(const DevSys& d, const Params& P, int si, uint32_t ent, int ti, float qi,
                                           float rc2, float rq2, float irc, float gmax, const PairCoef* pc,
                                           const float* us, const float* qt, uint4 qi4, const float (&fs)[3], Fix& fx,
                                           Fix& fy, Fix& fz, Fix& fu, Fix& fw) {
    const int sj = (int)(ent & kIdxMask);
    const int cls = (int)(ent >> kClassShift);
    const uint4 qj4 = d.pqs[sj];
    const float dx = __int2float_rn((int)(qi4.x - qj4.x)) * fs[0];
    const float dy = __int2float_rn((int)(qi4.y - qj4.y)) * fs[1];
    const float dz = __int2float_rn((int)(qi4.z - qj4.z)) * fs[2];
    const int tj = (int)qj4.w;
    const float r2 = dx * dx + dy * dy + dz * dz;
    const float ir = rsqrtf(r2);
    const float ir2 = ir * ir;
    const bool live = r2 >= 1e-6f;
    float g = 0.0f, u = 0.0f;
    if(SR) {
        const int pr = ti * P.T + tj;
        if(pc) {
            const PairCoef c = pc[pr];
            if(c.own2 < 0.0f) {
                if(live && r2 < rc2) pair_terms<float>(d, pr, r2, ir, ir2, g, u, ENERGY, P.lj_shift);
            } else {
                const bool in = live && r2 < fminf(rc2, c.own2);
                const float ir6 = ir2 * ir2 * ir2;
                const float t12 = c.a * ir6 * ir6, t6 = c.b * ir6;
                const float gl = (12.0f * t12 - 6.0f * t6) * ir2 - c.fs * ir;
                g = in ? gl : 0.0f;
                if(ENERGY) u = in ? t12 - t6 - us[pr] + r2 * ir * c.fs : 0.0f;
            }
        } else if(live && r2 < rc2) {
            pair_terms<float>(d, pr, r2, ir, ir2, g, u, ENERGY, P.lj_shift);
        }
    }
    if(P.qon) {
        const float qq = kCoulombKf * qi * (qt ? qt[tj] : d.qf[d.pcell_list[sj]]);
        const bool inq = live && r2 < rq2;
        float gq, uq = 0.0f;
        if(P.coulomb == MTG_COULOMB_SHIFTED) {
            gq = qq * (ir2 - irc * irc) * ir;
            if(ENERGY) uq = qq * (ir - irc + (r2 * ir - 1.0f / irc) * irc * irc);
        } else {
            gq = qq * ir2 * ir;
            if(ENERGY) uq = qq * ir;
        }
        g += inq ? gq : 0.0f;
        if(ENERGY) u += inq ? uq : 0.0f;
    }
    if(cls) {
        const float sc = P.scale[cls];
        g *= sc;
        u *= sc;
    }
    const float gc = fminf(fmaxf(g, -gmax), gmax);
    const float g16 = __fmul_rn(gc, 16.0f);
    fix_add16(fx, __fmul_rn(g16, dx));
    fix_add16(fy, __fmul_rn(g16, dy));
    fix_add16(fz, __fmul_rn(g16, dz));
    if(ENERGY && sj > si) {
        fix_add_clamped(fu, u);
        fix_add_clamped(fw, gc * r2);   // the pair's virial (r_i - r_j) . F_i, once per pair
    }
}

// Force gather: TEAM lanes per atom (8, 16 or 32; chosen per system by the autotuner), atoms taken
// in cell (slot) order so that a block's neighbour gathers stay within a compact, cache-resident
// range of the slot-ordered positions; each lane walks its share of the row four entries at a time
// so that four gathers are in flight per lane.  Bonded terms of the atom are spread over the
// team's lanes.  Mixed: every contribution is rounded to the 2^-26 fixed-point grid and summed as
// an integer, so forces do not depend on the team size, on the list order or on out-of-range
// list entries.  The FP64 form gets up to 80 registers (three blocks per SM): with 64 its four
// in-flight double-precision pairs spilled about 250 bytes per thread.
template<bool MIXED, bool ENERGY, int TEAM>
__global__ void __launch_bounds__(256, MIXED ? 4 : 3) k_pforce(DevSys d, Params P) {
    pdl_enter();
    using R = typename std::conditional<MIXED, float, double>::type;
    __shared__ PairCoef pc_s[kSmemPairs];
    __shared__ float us_s[kSmemPairs];   // energy shift of the staged LJ term
    __shared__ float qt_s[8];            // per-type charges (when charges are a function of type)
    const PairCoef* pc = nullptr;
    const float* qt = nullptr;
    if(MIXED && P.T * P.T <= kSmemPairs) {
        for(int q = threadIdx.x; q < P.T * P.T; q += blockDim.x) {
            PairCoef c{0.0f, 0.0f, 0.0f, 0.0f};
            float us = 0.0f;
            const int cnt = d.nb_cnt[q];
            if(cnt == 1 && d.nb_kind[q * kMaxFF] == MTG_NB_LJ) {
                const float4 f = reinterpret_cast<const float4*>(d.nb_parf)[q * kMaxFF];
                c = PairCoef{f.x, f.y, f.z > 0.0f ? f.z : FLT_MAX, P.lj_shift == 2 ? d.nb_fsf[q * kMaxFF] : 0.0f};
                us = f.w;
            } else if(cnt > 0) {
                c.own2 = -1.0f;
            }
            pc_s[q] = c;
            us_s[q] = us;
        }
        if(P.qtype && threadIdx.x < P.T) qt_s[threadIdx.x] = d.qtype[threadIdx.x];
        __syncthreads();
        pc = pc_s;
        if(P.qtype) qt = qt_s;
    }
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int si = gt / TEAM, lane = gt % TEAM;
    const bool active = si < P.n;
    const int i = active ? d.pcell_list[si] : 0;
    const bool mob = active && d.mobile[i] != 0;
    Fix fx{0, 0}, fy{0, 0}, fz{0, 0}, fu{0, 0}, fw{0, 0};   // mixed: exact fixed point
    double bx = 0, by = 0, bz = 0, bu = 0, bw = 0;          // fp64
    if(mob) {
        const SysView v = sys_view(d, P, rep_of_atom(d, P, i));
        const R rc2 = (R)v.rc * (R)v.rc;
        const R rq2 = (R)v.rcoul * (R)v.rcoul;
        const R irc = R(1) / (R)v.rcoul;
        const int cnt = min(d.vcount[si], d.vmax);   // an overflowed build is redone; stay in the row
        const uint32_t* lst = d.vlist + (size_t)si * d.vmax;
        if constexpr(MIXED) {
            const float fs[3] = {v.fscale[0], v.fscale[1], v.fscale[2]};
            const float gmax = 262143.0f / (v.rc + v.rcoul + v.skin);   // |d| < rc + rcoul + skin
            const uint4 qi4 = d.pqs[si];
            const int ti = (int)qi4.w;
            const float qi = d.qf[i];
            const int nsr = min(d.vsr[si], cnt);
            // the row's pairs with short-range terms, then (with charges on) its Coulomb-only pairs
            int e = lane;
            for(; e + 3 * TEAM < nsr; e += 4 * TEAM) {
                uint32_t ent[4];
#pragma unroll
                for(int q = 0; q < 4; q++) ent[q] = __ldg(lst + e + q * TEAM);
#pragma unroll
                for(int q = 0; q < 4; q++)
                    pair_mixed<ENERGY, true>(d, P, si, ent[q], ti, qi, rc2, rq2, irc, gmax, pc, us_s, qt, qi4, fs, fx, fy, fz, fu, fw);
            }
            for(; e < nsr; e += TEAM)
                pair_mixed<ENERGY, true>(d, P, si, __ldg(lst + e), ti, qi, rc2, rq2, irc, gmax, pc, us_s, qt, qi4, fs, fx, fy, fz, fu, fw);
            if(P.qon) {
                e = nsr + lane;
                for(; e + 3 * TEAM < cnt; e += 4 * TEAM) {
                    uint32_t ent[4];
#pragma unroll
                    for(int q = 0; q < 4; q++) ent[q] = __ldg(lst + e + q * TEAM);
#pragma unroll
                    for(int q = 0; q < 4; q++)
                        pair_mixed<ENERGY, false>(d, P, si, ent[q], ti, qi, rc2, rq2, irc, gmax, pc, us_s, qt, qi4, fs, fx, fy, fz, fu, fw);
                }
                for(; e < cnt; e += TEAM)
                    pair_mixed<ENERGY, false>(d, P, si, __ldg(lst + e), ti, qi, rc2, rq2, irc, gmax, pc, us_s, qt, qi4, fs, fx, fy, fz, fu, fw);
            }
        } else {
            const int ti = d.type[i];
            const double qi = d.qd[i];
            const double ri[3] = {d.r[3 * i], d.r[3 * i + 1], d.r[3 * i + 2]};
            const double L[3] = {v.box[0], v.box[1], v.box[2]};
            const double iL[3] = {1.0 / v.box[0], 1.0 / v.box[1], 1.0 / v.box[2]};
            // list entries name slots; the FP64 path works on atom indices
            auto atom_entry = [&](uint32_t ent) -> uint32_t {
                return (uint32_t)d.pcell_list[ent & kIdxMask] | (ent & ~kIdxMask);
            };
            int e = lane;
            for(; e + 3 * TEAM < cnt; e += 4 * TEAM) {
                uint32_t ent[4];
#pragma unroll
                for(int q = 0; q < 4; q++) ent[q] = atom_entry(__ldg(lst + e + q * TEAM));
#pragma unroll
                for(int q = 0; q < 4; q++) {
                    double dx, dy, dz, g, u;
                    pair_entry_d<ENERGY>(d, P, i, ent[q], ti, qi, rc2, rq2, irc, ri, L, iL, dx, dy, dz, g, u);
                    bx += g * dx; by += g * dy; bz += g * dz;
                    if(ENERGY) {
                        bu += u;
                        if((int)(ent[q] & kIdxMask) > i) bw += g * (dx * dx + dy * dy + dz * dz);
                    }
                }
            }
            for(; e < cnt; e += TEAM) {
                double dx, dy, dz, g, u;
                const uint32_t ent = atom_entry(__ldg(lst + e));
                pair_entry_d<ENERGY>(d, P, i, ent, ti, qi, rc2, rq2, irc, ri, L, iL, dx, dy, dz, g, u);
                bx += g * dx; by += g * dy; bz += g * dz;
                if(ENERGY) {
                    bu += u;
                    if((int)(ent & kIdxMask) > i) bw += g * (dx * dx + dy * dy + dz * dz);
                }
            }
        }
        // bonded terms of atom i, one entry per lane
        const int nbd = (d.bptr[i + 1] - d.bptr[i]) + (d.aptr[i + 1] - d.aptr[i]) + (d.dptr[i + 1] - d.dptr[i]);
        for(int b = lane; b < nbd; b += TEAM) {
            R gx = 0, gy = 0, gz = 0, gu = 0, gw = 0;
            bonded_entry<MIXED, R>(d, P, i, b, gx, gy, gz, gu, gw, ENERGY);
            if(MIXED) {
                fix_add_clamped(fx, (float)gx);
                fix_add_clamped(fy, (float)gy);
                fix_add_clamped(fz, (float)gz);
                if(ENERGY) {
                    fix_add_clamped(fu, (float)gu);
                    fix_add_clamped(fw, (float)gw);
                }
            } else {
                bx += (double)gx; by += (double)gy; bz += (double)gz;
                if(ENERGY) {
                    bu += (double)gu;
                    bw += (double)gw;
                }
            }
        }
    }
    // team reduction (integer: exact; FP64: fixed tree); teams are aligned within the warp
    if(MIXED) {
        long long ax = fix_total(fx), ay = fix_total(fy), az = fix_total(fz), au = ENERGY ? fix_total(fu) : 0;
        long long aw = ENERGY ? fix_total(fw) : 0;
        for(int o = TEAM / 2; o > 0; o >>= 1) {
            ax += __shfl_xor_sync(0xffffffffu, ax, o);
            ay += __shfl_xor_sync(0xffffffffu, ay, o);
            az += __shfl_xor_sync(0xffffffffu, az, o);
            if(ENERGY) {
                au += __shfl_xor_sync(0xffffffffu, au, o);
                aw += __shfl_xor_sync(0xffffffffu, aw, o);
            }
        }
        if(active && lane == 0) {
            d.Fx[i] = ax;
            d.Fy[i] = ay;
            d.Fz[i] = az;
            if(ENERGY) {
                d.U[i] = double(au) * (1.0 / kFixScale);
                d.W[i] = double(aw) * (1.0 / kFixScale);
            }
        }
    } else {
        for(int o = TEAM / 2; o > 0; o >>= 1) {
            bx += __shfl_xor_sync(0xffffffffu, bx, o);
            by += __shfl_xor_sync(0xffffffffu, by, o);
            bz += __shfl_xor_sync(0xffffffffu, bz, o);
            if(ENERGY) {
                bu += __shfl_xor_sync(0xffffffffu, bu, o);
                bw += __shfl_xor_sync(0xffffffffu, bw, o);
            }
        }
        if(active && lane == 0) {
            d.F[3 * i] = bx;
            d.F[3 * i + 1] = by;
            d.F[3 * i + 2] = bz;
            if(ENERGY) {
                d.U[i] = bu;
                d.W[i] = bw;
            }
        }
    }
}

// Conversions between the mixed-mode position/force formats and the FP64 host-facing arrays.
// Master FP64 arrays <-> mixed-mode mirrors (SyncMode).  From the masters the box fractions are
// computed by frac32_df, the same function the drift uses, so a round trip leaves them unchanged.
__global__ void k_sync(DevSys d, Params P, int mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n) return;
    if(mode == kSyncToMaster) {
        const float4 h = d.hi[i], l = d.lo[i], ph = d.ph[i], pl = d.pl[i];
        d.r[3 * i] = (double)h.x + (double)l.x;
        d.r[3 * i + 1] = (double)h.y + (double)l.y;
        d.r[3 * i + 2] = (double)h.z + (double)l.z;
        d.p[3 * i] = (double)ph.x + (double)pl.x;
        d.p[3 * i + 1] = (double)ph.y + (double)pl.y;
        d.p[3 * i + 2] = (double)ph.z + (double)pl.z;
        return;
    }
    const SysView v = sys_view(d, P, rep_of_atom(d, P, i));
    const DF x = df_of(d.r[3 * i]), y = df_of(d.r[3 * i + 1]), z = df_of(d.r[3 * i + 2]);
    d.hi[i] = make_float4(x.h, y.h, z.h, d.qf[i]);
    d.lo[i] = make_float4(x.l, y.l, z.l, __int_as_float(d.type[i]));
    const uint4 qi = make_uint4(frac32_df(x, df_of(v.fconv[0])), frac32_df(y, df_of(v.fconv[1])),
                                frac32_df(z, df_of(v.fconv[2])), (unsigned int)d.type[i]);
    d.pq[i] = qi;
    d.pqs[d.slot_of[i]] = qi;
    if(mode == kSyncFromMaster) {
        const DF px = df_of(d.p[3 * i]), py = df_of(d.p[3 * i + 1]), pz = df_of(d.p[3 * i + 2]);
        const DF im = df_of(1.0 / d.m[i]);
        d.ph[i] = make_float4(px.h, py.h, pz.h, im.h);
        d.pl[i] = make_float4(px.l, py.l, pz.l, im.l);
    }
}

__global__ void k_forces_to_double(DevSys d, Params P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n) return;
    d.F[3 * i] = double(d.Fx[i]) * (1.0 / kFixScale);
    d.F[3 * i + 1] = double(d.Fy[i]) * (1.0 / kFixScale);
    d.F[3 * i + 2] = double(d.Fz[i]) * (1.0 / kFixScale);
}

// State after the completed step, on the device (no host round trip).  The kernels apply the
// thermostat's second-half scale c2 of a step lazily at the next kick; these bring the momenta up
// to it (mixed: the FP64 master is (hi + lo) c2 rounded to the nearest double-float, which the
// mirrors then hold), rewind the chains to their state after the second half-step and, under NPT,
// the barostat to the completed step (its box fields recomputed for that box).
__global__ void k_settle_momenta(DevSys d, Params P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if(i >= P.n) return;
    const double c2 = P.nrep ? d.rsc[d.rep_of[i]].c2 : d.sc->c2;
    if(c2 == 1.0) return;
    if(P.precision == MTG_PREC_MIXED) {
        const float4 ph = d.ph[i], pl = d.pl[i];
        const DF x = df_of(((double)ph.x + (double)pl.x) * c2);
        const DF y = df_of(((double)ph.y + (double)pl.y) * c2);
        const DF z = df_of(((double)ph.z + (double)pl.z) * c2);
        d.ph[i] = make_float4(x.h, y.h, z.h, ph.w);
        d.pl[i] = make_float4(x.l, y.l, z.l, pl.w);
        d.p[3 * i] = (double)x.h + (double)x.l;
        d.p[3 * i + 1] = (double)y.h + (double)y.l;
        d.p[3 * i + 2] = (double)z.h + (double)z.l;
    } else {
        d.p[3 * i] *= c2;
        d.p[3 * i + 1] *= c2;
        d.p[3 * i + 2] *= c2;
    }
}

__global__ void k_settle_scalars(DevSys d, Params P) {
    if(P.nrep) {
        for(int r = threadIdx.x; r < P.nrep; r += blockDim.x) {
            StepScalars& s = d.rsc[r];
            if(s.c2 != 1.0 || s.S != 1.0) {
                d.ths[r] = d.ths_saved[r];
                s.c2 = 1.0;
                s.S = 1.0;
            }
        }
        return;
    }
    if(threadIdx.x != 0) return;
    StepScalars* s = d.sc;
    if(s->c2 != 1.0 || s->S != 1.0) {
        *d.th = *d.th_saved;
        s->c2 = 1.0;
        s->S = 1.0;
    }
    if(P.ensemble == MTG_NPT) {
        BaroDev& b = *d.baro;
        b.p_eps = b.p_eps_saved;
        b.eps = b.eps_saved;
        for(int a = 0; a < 3; a++) {
            b.L[a] = b.L_saved[a];
            b.Lf[a] = (float)b.L[a];
        }
        if(P.precision != MTG_PREC_REFERENCE) baro_box_fields(P, b);
        *d.thp = *d.thp_saved;
    }
}

__global__ void k_set_chains(DevSys d, ChainSet cs) {
    if(threadIdx.x != 0) return;
    for(int j = 0; j < cs.M; j++) {
        d.th->eta[j] = d.th_saved->eta[j] = cs.eta[j];
        d.th->peta[j] = d.th_saved->peta[j] = cs.peta[j];
    }
    if(cs.set_baro) {
        for(int j = 0; j < cs.MP; j++) {
            d.thp->eta[j] = d.thp_saved->eta[j] = cs.etaP[j];
            d.thp->peta[j] = d.thp_saved->peta[j] = cs.petaP[j];
        }
        *d.baro = cs.baro;
    }
}

// Positions written from the host (FP64 masters; mixed mode has synced its mirrors): flags a list
// rebuild when an atom lies more than half the skin from its position at the last build, the
// test the kick-drift applies every step (the box does not change here).
__global__ void k_check_list(DevSys d, Params P) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= P.n) return;
    const SysView v = sys_view(d, P, rep_of_atom(d, P, k));
    const double h = 0.5 * double(v.skin);
    double d2 = 0.0;
#pragma unroll
    for(int a = 0; a < 3; a++) {
        const double x = minimg_d(d.r[3 * k + a] - d.r_build[3 * k + a], v.box[a], 1.0 / v.box[a]);
        d2 += x * x;
    }
    if(d2 > h * h) flag_rebuild(d, P, v);
}

// End of a list build: the cell counts go back to zero for the next build (they start at zero
// when allocated), and the last block clears the rebuild flags and counts the build.  Every block
// passes the early-exit test before the last one clears the flag it tests.
__global__ void k_finish_build(DevSys d, Params P, int ncell) {
    pdl_enter();
    if(!d.sc->rebuild) return;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if(c < ncell) d.pcell_count[c] = 0;
    if(last_block(&d.sc->done_blocks)) {
        for(int r = threadIdx.x; r < P.nrep; r += blockDim.x) d.rsc[r].rebuild = 0;
        __syncthreads();
        if(threadIdx.x == 0) {
            d.sc->done_blocks = 0;
            d.sc->rebuild = 0;
            d.sc->builds += 1;
            d.sc->builds_run += 1;
        }
    }
}

// Gradient-descent step of CSimulationBox::gradientDescentStep (SimulationBox.cpp:197-208):
// r += lr F, no clipping, no wrapping.  Also sums U, p^2/m and F.r (after the move) for the
// output line, and flags a production list rebuild when an atom moved beyond skin/2.
__global__ void k_gd_step(DevSys d, Params P, double lr, int mode) {
    __shared__ double smem[32 * 3];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0.0, 0.0, 0.0};
    const SysView sv = sys_view(d, P, -1);   // the current box (it changes under NPT)
    if(k < P.n) {
        const bool mixed = (mode == MTG_PREC_MIXED);
        double f[3], r[3];
        load_force(d, k, f[0], f[1], f[2], mixed);
        load_pos(d, k, r[0], r[1], r[2], mixed);
        double pk[3] = {d.p[3 * k], d.p[3 * k + 1], d.p[3 * k + 2]};
        if(mixed) {   // the double-float mirrors are current
            const float4 h = d.ph[k], l = d.pl[k];
            pk[0] = (double)h.x + (double)l.x;
            pk[1] = (double)h.y + (double)l.y;
            pk[2] = (double)h.z + (double)l.z;
        }
        double fr = 0.0, p2 = 0.0;
        for(int a = 0; a < 3; a++) {
            r[a] = r[a] + f[a] * lr;
            fr += f[a] * r[a];
            p2 += pk[a] * pk[a];
        }
        store_pos(d, sv.fconv, k, r[0], r[1], r[2], mixed);
        if(mode != MTG_PREC_REFERENCE) {
            const bool npt = P.ensemble == MTG_NPT;
            const double sb = npt ? (double)d.baro->sb : 1.0;
            const double h = 0.5 * double(P.skin);
            const double h2 = npt ? (double)d.baro->h2 : h * h;
            const double bx = minimg_d(r[0] - d.r_build[3 * k] * sb, sv.box[0], 1.0 / sv.box[0]);
            const double by = minimg_d(r[1] - d.r_build[3 * k + 1] * sb, sv.box[1], 1.0 / sv.box[1]);
            const double bz = minimg_d(r[2] - d.r_build[3 * k + 2] * sb, sv.box[2], 1.0 / sv.box[2]);
            if(bx * bx + by * by + bz * bz > h2) d.sc->rebuild = -1;
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
            const double V = sv.box[0] * sv.box[1] * sv.box[2];
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

void set_pdl_launch(bool on) { g_pdl = on; }

void launch_prologue(const DevSys& d, const Params& P, cudaStream_t s) {
    if(P.precision == MTG_PREC_MIXED) k_prologue<true><<<integration_blocks(P), 256, 0, s>>>(d, P);
    else k_prologue<false><<<integration_blocks(P), 256, 0, s>>>(d, P);
}

void launch_prod_kick_drift(const DevSys& d, const Params& P, cudaStream_t s, cudaGraphConditionalHandle cond, bool use_cond) {
    const int nb = integration_blocks(P);
    const int u = use_cond ? 1 : 0;
    if(P.precision == MTG_PREC_MIXED && P.ensemble == MTG_NPT) launch_step_kernel(k_mkick_drift_npt, nb, 256, s, d, P, cond, u);
    else if(P.precision == MTG_PREC_MIXED) launch_step_kernel(k_mkick_drift, nb, 256, s, d, P, cond, u);
    else launch_step_kernel(k_pkick_drift, nb, 256, s, d, P, cond, u);
}

void launch_prod_check_list(const DevSys& d, const Params& P, cudaStream_t s) {
    k_check_list<<<nblk(P.n, 256), 256, 0, s>>>(d, P);
}

void launch_prod_build(const DevSys& d, const Params& P, bool force, cudaStream_t s) {
    const int ncell = P.nrep ? P.ncell_total : P.pnx * P.pny * P.pnz;
    if(force) cudaMemsetAsync(&d.sc->rebuild, 0xff, sizeof(int32_t), s);
    // the cell counts are zero here (k_finish_build); every kernel returns at once when no
    // rebuild is due
    if(P.precision == MTG_PREC_MIXED) launch_step_kernel(k_pcell_assign<true>, nblk(P.n, 256), 256, s, d, P);
    else launch_step_kernel(k_pcell_assign<false>, nblk(P.n, 256), 256, s, d, P);
    launch_step_kernel(k_pcell_scan, P.nrep ? P.nrep : 1, 1024, s, d, P);
    launch_step_kernel(k_pcell_scatter, nblk(P.n, 256), 256, s, d, P);
    launch_step_kernel(k_pcell_rank, nblk(P.n, 256), 256, s, d, P, P.precision == MTG_PREC_MIXED);
    if(P.precision == MTG_PREC_MIXED) launch_step_kernel(k_vlist<true>, nblk(P.n * 32, 256), 256, s, d, P);
    else launch_step_kernel(k_vlist<false>, nblk(P.n * 32, 256), 256, s, d, P);
    launch_step_kernel(k_finish_build, nblk(ncell, 256), 256, s, d, P, ncell);
}

template<bool MIXED, bool ENERGY>
static void force_team(const DevSys& d, const Params& P, cudaStream_t s) {
    const int team = P.team;
    const int nb = nblk(P.n * team, 256);
    if(team == 8) launch_step_kernel(k_pforce<MIXED, ENERGY, 8>, nb, 256, s, d, P);
    else if(team == 16) launch_step_kernel(k_pforce<MIXED, ENERGY, 16>, nb, 256, s, d, P);
    else launch_step_kernel(k_pforce<MIXED, ENERGY, 32>, nb, 256, s, d, P);
}

void launch_prod_force(const DevSys& d, const Params& P, bool energy, cudaStream_t s) {
    energy = energy || P.ensemble == MTG_NPT;   // the energy variant also sums the virial
    if(P.precision == MTG_PREC_MIXED) {
        if(energy) force_team<true, true>(d, P, s);
        else force_team<true, false>(d, P, s);
    } else {
        if(energy) force_team<false, true>(d, P, s);
        else force_team<false, false>(d, P, s);
    }
}

void launch_prod_kick2(const DevSys& d, const Params& P, bool output, cudaStream_t s, int parts) {
    const int nb = integration_blocks(P);
    if(P.precision == MTG_PREC_MIXED) {
        const int nsys = P.nrep ? P.nrep : 1;
        if((parts & kKick2Atoms) && P.ensemble == MTG_NPT) {
            if(output) launch_step_kernel(k_mkick2_npt<true>, nb, 256, s, d, P);
            else launch_step_kernel(k_mkick2_npt<false>, nb, 256, s, d, P);
        } else if(parts & kKick2Atoms) {
            if(output) launch_step_kernel(k_mkick2<true>, nb, 256, s, d, P);
            else launch_step_kernel(k_mkick2<false>, nb, 256, s, d, P);
        }
        if((parts & kKick2StepEnd) && P.ensemble == MTG_NPT) {
            if(output) launch_step_kernel(k_mstep_end_npt<true>, 1, 96, s, d, P);
            else launch_step_kernel(k_mstep_end_npt<false>, 1, 96, s, d, P);
        } else if(parts & kKick2StepEnd) {
            if(output) launch_step_kernel(k_mstep_end<true>, nsys, 96, s, d, P);
            else launch_step_kernel(k_mstep_end<false>, nsys, 96, s, d, P);
        }
    } else if(parts & kKick2Atoms) {
        if(output) launch_step_kernel(k_pkick2<true>, nb, 256, s, d, P);
        else launch_step_kernel(k_pkick2<false>, nb, 256, s, d, P);
    }
}

void launch_settle(const DevSys& d, const Params& P, cudaStream_t s) {
    if(P.precision == MTG_PREC_MIXED) k_sync<<<nblk(P.n, 256), 256, 0, s>>>(d, P, (int)kSyncToMaster);
    k_settle_momenta<<<nblk(P.n, 256), 256, 0, s>>>(d, P);
    k_settle_scalars<<<1, 256, 0, s>>>(d, P);
}

void launch_set_chains(const DevSys& d, const ChainSet& cs, cudaStream_t s) { k_set_chains<<<1, 32, 0, s>>>(d, cs); }

__global__ void k_copy_table(CopyTable t) {
    // block y = copy, blocks x stride over its words
    const int q = blockIdx.y;
    if(q >= t.n) return;
    const unsigned long long* src = t.src[q];
    unsigned long long* dst = t.dst[q];
    for(unsigned long long w = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; w < t.words[q];
        w += (unsigned long long)gridDim.x * blockDim.x)
        dst[w] = src[w];
}

void launch_copy_table(const CopyTable& t, cudaStream_t s) {
    if(t.n <= 0) return;
    unsigned long long most = 0;
    for(int q = 0; q < t.n; q++) most = t.words[q] > most ? t.words[q] : most;
    const int bx = (int)((most + 255) / 256 < 304 ? (most + 255) / 256 : 304);
    k_copy_table<<<dim3(bx > 0 ? bx : 1, t.n), 256, 0, s>>>(t);
}

void launch_prod_sync(const DevSys& d, const Params& P, SyncMode mode, cudaStream_t s) {
    k_sync<<<nblk(P.n, 256), 256, 0, s>>>(d, P, (int)mode);
}

void launch_prod_forces_to_double(const DevSys& d, const Params& P, cudaStream_t s) {
    k_forces_to_double<<<nblk(P.n, 256), 256, 0, s>>>(d, P);
}

}  // namespace mtg
