// Device helpers shared by the reference-mode and production kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mtg_internal.h"

namespace mtg {

// exp(x) for the thermostat.  Small arguments, which are the normal case (|x| = Dt/8 p_eta/Q is of
// order 1e-2), use the Taylor series of e^x with the remainder below 1e-17 relative (degree 8 for
// |x| <= 2^-5, degree 11 for |x| <= 2^-3); larger ones call exp().  On this GPU every FP64
// instruction costs about as much as thirty FP32 ones, so the instruction count is what matters.
__device__ __forceinline__ double nh_exp(double x) {
    const double ax = fabs(x);
    if(ax <= 0.03125) {
        double p = 1.0 / 40320.0;
        p = fma(p, x, 1.0 / 5040.0);
        p = fma(p, x, 1.0 / 720.0);
        p = fma(p, x, 1.0 / 120.0);
        p = fma(p, x, 1.0 / 24.0);
        p = fma(p, x, 1.0 / 6.0);
        p = fma(p, x, 0.5);
        p = fma(p, x, 1.0);
        return fma(p, x, 1.0);
    }
    if(ax <= 0.125) {
        double p = 1.0 / 39916800.0;
        p = fma(p, x, 1.0 / 3628800.0);
        p = fma(p, x, 1.0 / 362880.0);
        p = fma(p, x, 1.0 / 40320.0);
        p = fma(p, x, 1.0 / 5040.0);
        p = fma(p, x, 1.0 / 720.0);
        p = fma(p, x, 1.0 / 120.0);
        p = fma(p, x, 1.0 / 24.0);
        p = fma(p, x, 1.0 / 6.0);
        p = fma(p, x, 0.5);
        p = fma(p, x, 1.0);
        return fma(p, x, 1.0);
    }
    return exp(x);
}

// CMt::exp (Integrators/Math.cpp:29-38): linear above x = 1.
__device__ __forceinline__ double cmt_exp(double x) { return (x > 1.0) ? 2.71828 * x : nh_exp(x); }

// One call of CNHChain::propagator with the thermostat functor CFctT (NHChain.cpp:54-113,
// MDLoop.cpp:29-60), executed by all 32 lanes of one warp.  The particles enter only through
// G(0) = sum p^2/m - g kT and through the momentum scalings; since a scaling by c multiplies
// sum p^2/m by c^2, the kinetic term is carried as the scalar `KE2` and the scalings are returned
// as one product.  Every lane carries the whole chain (the serial recurrences run redundantly);
// work that is independent across chain elements -- the exponentials of step 1.2 and the eta
// updates of step 1.3 -- is spread over lanes, so it costs one instruction stream, not M.
// The two identical exponentials of each update (NHChain.cpp:72-78, 92-98) are evaluated once, and
// 1/Q_j comes precomputed in th.iQ.  Suzuki-Yoshida weights as the reference sets them:
// w0 = 1/(1 - 2^(1/3)) (NHChain.cpp:45-52).  Lane j writes eta[j] and peta[j] back.
__device__ inline double nh_chain_half(ThermoDev& th, double& KE2, double g, double kT, double dt, int M, int nresp) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const double w0 = 1.0 / (1.0 - cbrt(2.0));
    const double w[3] = {w0, 1.0 - 2.0 * w0, w0};
    double scale = 1.0;
    if(M <= 0) return scale;
    double pe[kMaxChain], iQ[kMaxChain];
    for(int j = 0; j < M; j++) {
        pe[j] = th.peta[j];
        iQ[j] = th.iQ[j];
    }
    double eta_mine = (lane < M) ? th.eta[lane] : 0.0;
    const double gkT = g * kT;
    if(pe[0] > 15.0) pe[0] = 10.0;
    for(int mu = 0; mu < 3; mu++) {
        const double Dt = w[mu] * dt / double(nresp);
        const double d8 = -(Dt / 8.0), d4 = Dt / 4.0, d2 = Dt / 2.0;
        for(int it = 0; it < nresp; it++) {
            // 1.1
            pe[M - 1] += d4 * ((M - 1 == 0) ? KE2 - gkT : pe[M - 2] * pe[M - 2] * iQ[M - 2] - kT);
            // 1.2: the exponentials use the chain as it stands (pe[M-1] just updated)
            double cl = 1.0;
            if(lane < M - 1) {
                double v = 0.0, q = 0.0;
                for(int j = 0; j < M - 1; j++)
                    if(j == lane) { v = pe[j + 1]; q = iQ[j + 1]; }
                cl = cmt_exp(d8 * (v * q));
            }
            double c_last = 1.0;
            for(int j = 0; j < M - 1; j++) {
                const double c = __shfl_sync(full, cl, j);
                const double G = (j == 0) ? KE2 - gkT : pe[j - 1] * pe[j - 1] * iQ[j - 1] - kT;
                pe[j] = (pe[j] * c + d4 * G) * c;
                c_last = c;
            }
            // 1.3
            {
                double v = 0.0, q = 0.0;
                for(int j = 0; j < M; j++)
                    if(j == lane) { v = pe[j]; q = iQ[j]; }
                if(lane < M) eta_mine += d2 * (v * q);
            }
            // 1.4
            {
                const double c = cmt_exp(-(d2 * (pe[0] * iQ[0])));
                scale *= c;
                KE2 *= c * c;
            }
            // 1.5 (the first update reuses the exponential of pe[M-1], unchanged since 1.2)
            for(int j = M - 2; j >= 0; j--) {
                const double c = (j == M - 2) ? c_last : cmt_exp(d8 * (pe[j + 1] * iQ[j + 1]));
                const double G = (j == 0) ? KE2 - gkT : pe[j - 1] * pe[j - 1] * iQ[j - 1] - kT;
                pe[j] = (pe[j] * c + d4 * G) * c;
            }
            // 1.6
            pe[M - 1] += d4 * ((M - 1 == 0) ? KE2 - gkT : pe[M - 2] * pe[M - 2] * iQ[M - 2] - kT);
        }
    }
    __syncwarp(full);
    if(lane < M) {
        double v = 0.0;
        for(int j = 0; j < M; j++)
            if(j == lane) v = pe[j];
        th.peta[lane] = v;
        th.eta[lane] = eta_mine;
    }
    __syncwarp(full);
    return scale;
}

// Deterministic block sum of NV doubles (fixed shuffle tree, then fixed order over warps).
template<int NV>
__device__ inline void block_sum(double (&v)[NV], double* smem /* [32*NV] */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for(int k = 0; k < NV; k++) {
        double x = v[k];
        for(int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if(lane == 0) smem[warp * NV + k] = x;
    }
    __syncthreads();
    if(threadIdx.x == 0) {
#pragma unroll
        for(int k = 0; k < NV; k++) {
            double s = 0.0;
            for(int w = 0; w < nw; w++) s += smem[w * NV + k];
            v[k] = s;
        }
    }
    __syncthreads();
}

// Last-block election: every block stores its partials, fences, and bumps the counter; the block
// that observes the final count reads all partials (in block order) and resets the counter.
__device__ inline bool last_block(unsigned int* counter) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if(threadIdx.x == 0) {
        unsigned int prev = atomicAdd(counter, 1u);
        is_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if(is_last) __threadfence();
    return is_last;
}

// End-of-step scalar work of the last block, run by its warp 0 (all lanes): the second
// thermostat half-step of this step and the first half-step of the next one (MDLoop.cpp:129-132);
// record output scalars when asked.  The chain state is shared through `th` in global memory;
// lanes read it, each lane j writes element j back.
__device__ inline void end_of_step(const Params& P, StepScalars* sc, ThermoDev* th, ThermoDev* th_saved,
                                   double KE2, double U, double vir, bool output, double* rec) {
    const int lane = threadIdx.x & 31;
    const double g = double(3 * P.n);
    double c2 = 1.0, c1 = 1.0;
    if(P.ensemble == MTG_NVT || P.ensemble == MTG_NPT) {
        c2 = nh_chain_half(*th, KE2, g, P.kT, P.dt, P.M, P.nresp);
        __threadfence_block();
        if(lane < P.M) {
            th_saved->eta[lane] = th->eta[lane];
            th_saved->peta[lane] = th->peta[lane];
        }
        __syncwarp();
        double KEn = KE2;
        c1 = nh_chain_half(*th, KEn, g, P.kT, P.dt, P.M, P.nresp);
    }
    if(lane == 0) {
        sc->c2 = c2;
        sc->S = c2 * c1;
        sc->KE2 = KE2;
        if(output) {
            const double V = P.box[0] * P.box[1] * P.box[2];
            // MDLoop.cpp:388-403 / SimulationBox.cpp:168-195: T = sum p^2/m / 3N, P = (sum p^2/m + sum F.r)/3V
            rec[0] = U;
            rec[1] = 0.5 * KE2;
            rec[2] = KE2 / (3.0 * double(P.n));
            rec[3] = (1.0 / (3.0 * V)) * (KE2 + vir);
            rec[4] = V;
            sc->U = U;
            sc->virial = vir;
        }
    }
}

// Minimum image by rounding (production kernels).
__device__ __forceinline__ float minimg_f(float d, float L, float invL) { return d - L * rintf(d * invL); }
__device__ __forceinline__ double minimg_d(double d, double L, double invL) { return d - L * rint(d * invL); }

}  // namespace mtg
