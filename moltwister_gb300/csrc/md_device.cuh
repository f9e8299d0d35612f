// Device helpers shared by the reference-mode and production kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mtg_internal.h"

namespace mtg {

// CMt::exp (Integrators/Math.cpp:29-38): linear above x = 1.
__device__ __forceinline__ double cmt_exp(double x) { return (x > 1.0) ? 2.71828 * x : exp(x); }

// One call of CNHChain::propagator with the thermostat functor CFctT (NHChain.cpp:54-113,
// MDLoop.cpp:29-60), single thread.  The particles enter only through G(0) = sum p^2/m - g kT and
// through the momentum scalings; since a scaling by c multiplies sum p^2/m by c^2, the kinetic
// term is carried as the scalar `KE2` (= sum p^2/m) and the scalings are returned as one product.
// Suzuki-Yoshida weights as the reference sets them: w0 = 1/(1 - 2^(1/3)) (NHChain.cpp:45-52).
__device__ inline double nh_chain_half(ThermoDev& th, double& KE2, double g, double kT, double dt, int M, int nresp) {
    const double w0 = 1.0 / (1.0 - pow(2.0, 1.0 / 3.0));
    const double w[3] = {w0, 1.0 - 2.0 * w0, w0};
    const double beta = 1.0 / kT;
    double scale = 1.0;
    if(M <= 0) return scale;
    if(th.peta[0] > 15.0) th.peta[0] = 10.0;
    double* pe = th.peta;
    const double* Q = th.Q;
    for(int mu = 0; mu < 3; mu++) {
        const double Dt = w[mu] * dt / double(nresp);
        for(int it = 0; it < nresp; it++) {
            // 1.1
            {
                const int j = M - 1;
                const double G = (j == 0) ? KE2 - (g / beta) : (pe[j - 1] * pe[j - 1] / Q[j - 1]) - (1.0 / beta);
                pe[j] += (Dt / 4.0) * G;
            }
            // 1.2
            for(int j = 0; j < M - 1; j++) {
                double c = cmt_exp(-(Dt / 8.0) * (pe[j + 1] / Q[j + 1]));
                pe[j] *= c;
                const double G = (j == 0) ? KE2 - (g / beta) : (pe[j - 1] * pe[j - 1] / Q[j - 1]) - (1.0 / beta);
                pe[j] += (Dt / 4.0) * G;
                c = cmt_exp(-(Dt / 8.0) * (pe[j + 1] / Q[j + 1]));
                pe[j] *= c;
            }
            // 1.3
            for(int j = 0; j < M; j++) th.eta[j] += (Dt / 2.0) * (pe[j] / Q[j]);
            // 1.4: scale momenta
            {
                const double c = cmt_exp(-((Dt / 2.0) * (pe[0] / Q[0])));
                scale *= c;
                KE2 *= c * c;
            }
            // 1.5
            for(int j = M - 2; j >= 0; j--) {
                double c = cmt_exp(-(Dt / 8.0) * (pe[j + 1] / Q[j + 1]));
                pe[j] *= c;
                const double G = (j == 0) ? KE2 - (g / beta) : (pe[j - 1] * pe[j - 1] / Q[j - 1]) - (1.0 / beta);
                pe[j] += (Dt / 4.0) * G;
                c = cmt_exp(-(Dt / 8.0) * (pe[j + 1] / Q[j + 1]));
                pe[j] *= c;
            }
            // 1.6
            {
                const int j = M - 1;
                const double G = (j == 0) ? KE2 - (g / beta) : (pe[j - 1] * pe[j - 1] / Q[j - 1]) - (1.0 / beta);
                pe[j] += (Dt / 4.0) * G;
            }
        }
    }
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

// End-of-step scalar work of the last block: the second thermostat half-step of this step and
// the first half-step of the next one (MDLoop.cpp:129-132); record output scalars when asked.
__device__ inline void end_of_step(const Params& P, StepScalars* sc, ThermoDev* th, ThermoDev* th_saved,
                                   double KE2, double U, double vir, bool output, double* rec) {
    const double g = double(3 * P.n);
    double c2 = 1.0, c1 = 1.0;
    if(P.ensemble == MTG_NVT || P.ensemble == MTG_NPT) {
        ThermoDev t = *th;
        c2 = nh_chain_half(t, KE2, g, P.kT, P.dt, P.M, P.nresp);
        *th_saved = t;
        double KEn = KE2;
        c1 = nh_chain_half(t, KEn, g, P.kT, P.dt, P.M, P.nresp);
        *th = t;
    }
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

// Minimum image by rounding (production kernels).
__device__ __forceinline__ float minimg_f(float d, float L, float invL) { return d - L * rintf(d * invL); }
__device__ __forceinline__ double minimg_d(double d, double L, double invL) { return d - L * rint(d * invL); }

}  // namespace mtg
