// Device helpers shared by the reference-mode and production kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mtg_internal.h"

namespace mtg {

// exp(x) for the thermostat.  Small arguments, which are the normal case (|x| = Dt/8 p_eta/Q is of
// order 1e-2), use the Taylor series of e^x with the remainder below 1e-17 relative (degree 8 for
// |x| <= 2^-5, degree 11 for |x| <= 2^-3); larger ones call exp().  On this GPU an FP64
// instruction costs about 100 cycles in the chain's warps whether or not it depends on the one
// before, so the instruction count is what matters: Horner's scheme (one FMA per degree;
// Estrin's shorter dependency chain needs more instructions and measured slower), the range
// tests compare bit patterns on the integer units, and the wider ranges sit in a function that
// is not inlined: inlined, their instructions could be predicated off but would still occupy the
// FP64 pipe on every call.
static __device__ __noinline__ double nh_exp_wide(double x);

__device__ __forceinline__ double nh_exp(double x) {
    const long long ax = __double_as_longlong(x) & 0x7fffffffffffffffLL;
    if(ax <= 0x3fa0000000000000LL) {            // |x| <= 2^-5
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
    return nh_exp_wide(x);
}

static __device__ __noinline__ double nh_exp_wide(double x) {
    const long long ax = __double_as_longlong(x) & 0x7fffffffffffffffLL;
    if(ax <= 0x3fc0000000000000LL) {            // |x| <= 2^-3
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

// The chain integrator's constants.  The reference (fixed = false) uses w0 = 1/(1 - 2^(1/3)) for
// its order-3 Suzuki-Yoshida weights (NHChain.cpp:45-52), CMt::exp and the clamp p_eta[0] > 15 ->
// 10 (NHChain.cpp:61-65).  With those, chains of large systems diverge: Q_0 grows with N while
// Q_j (j > 0) does not, so the upper chain velocities grow, the linear branch of CMt::exp breaks
// the cancellation between the negative and positive Suzuki-Yoshida stages, and p_eta[0] > 15 is
// the normal state of a large system.  The production modes (fixed = true) use the published
// weight w0 = 1/(2 - 2^(1/3)), the exponential itself and no clamp.
__device__ __forceinline__ double sy_w0(bool fixed) { return fixed ? 1.0 / (2.0 - cbrt(2.0)) : 1.0 / (1.0 - cbrt(2.0)); }
__device__ __forceinline__ double chain_exp(double x, bool fixed) { return fixed ? nh_exp(x) : cmt_exp(x); }

// One call of CNHChain::propagator with the thermostat functor CFctT (NHChain.cpp:54-113,
// MDLoop.cpp:29-60), executed by all 32 lanes of one warp.  The particles enter only through
// G(0) = sum p^2/m - g kT and through the momentum scalings; since a scaling by c multiplies
// sum p^2/m by c^2, the kinetic term is carried as the scalar `KE2` and the scalings are returned
// as one product.  Every lane carries the whole chain (the serial recurrences run redundantly);
// work that is independent across chain elements -- the exponentials of step 1.2 and the eta
// updates of step 1.3 -- is spread over lanes, so it costs one instruction stream, not M.
// The two identical exponentials of each update (NHChain.cpp:72-78, 92-98) are evaluated once, and
// 1/Q_j comes precomputed in th.iQ.  Suzuki-Yoshida weights, exponential and p_eta[0] clamp as
// sy_w0 / chain_exp describe (the reference's, or the published ones with `fixed`).  Lane j
// writes eta[j] and peta[j] back.
__device__ inline double nh_chain_half(ThermoDev& th, double& KE2, double g, double kT, double dt, int M, int nresp,
                                       bool fixed) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const double w0 = sy_w0(fixed);
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
    if(!fixed && pe[0] > 15.0) pe[0] = 10.0;
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
                cl = chain_exp(d8 * (v * q), fixed);
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
                const double c = chain_exp(-(d2 * (pe[0] * iQ[0])), fixed);
                scale *= c;
                KE2 *= c * c;
            }
            // 1.5 (the first update reuses the exponential of pe[M-1], unchanged since 1.2)
            for(int j = M - 2; j >= 0; j--) {
                const double c = (j == M - 2) ? c_last : chain_exp(d8 * (pe[j + 1] * iQ[j + 1]), fixed);
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

// ---------------------------------------------------------------------------------------------
// Double-float arithmetic for the mixed-mode integrator.  The FP64 unit of this GPU runs at a
// small fraction of the FP32 rate (64-bit conversions included), so per-atom FP64 work made the
// kick and drift kernels slower than the force gather at 10^6 atoms.  A value is the unevaluated
// sum h + l of two floats with |l| <= ulp(h)/2 (about 48 significant bits); the error-free
// transformations below are Knuth's two-sum, Dekker's fast two-sum and the FMA-based exact
// product.  The _rn intrinsics keep the compiler from contracting or reordering them.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ DF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ DF fast_two_sum(float a, float b) {   // |a| >= |b| (or a = 0)
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const DF s = two_sum(a.h, b.h);
    const DF t = two_sum(a.l, b.l);
    const DF u = fast_two_sum(s.h, __fadd_rn(s.l, t.h));
    return fast_two_sum(u.h, __fadd_rn(u.l, t.l));
}
__device__ __forceinline__ DF df_neg(DF a) { return {-a.h, -a.l}; }
__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const float p = __fmul_rn(a.h, b.h);
    const float c = __fmaf_rn(a.l, b.h, __fmul_rn(a.h, b.l));   // cross terms, beside p
    const float e = __fmaf_rn(a.h, b.h, -p);                    // exact error of p
    return fast_two_sum(p, __fadd_rn(e, c));
}
__device__ __forceinline__ DF df_mul_f(DF a, float b) {
    const float p = __fmul_rn(a.h, b);
    return fast_two_sum(p, __fmaf_rn(a.l, b, __fmaf_rn(a.h, b, -p)));
}
// FP64 <-> double-float (FP64 instructions: used once per block or outside the step loop)
__device__ __forceinline__ DF df_of(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double df_val(DF a) { return (double)a.h + (double)a.l; }
// Fixed-point force q (units 2^-26) as a double-float: q = a 2^22 + b with 0 <= b < 2^22, both
// parts converted by 32-bit conversions (exact for |q| < 2^46, i.e. |F| < 2^20 kJ/(mol A)).
__device__ __forceinline__ DF df_fix(long long q) {
    const int a = (int)(q >> 22);
    const int b = (int)(q & 0x3FFFFFLL);
    return two_sum(__fmul_rn(__int2float_rn(a), 0.0625f), __fmul_rn(__int2float_rn(b), 1.4901161193847656e-08f));
}
// Box fraction round(x * conv) modulo 2^32 (conv = 2^32 / L) from double-float operands, to
// within one unit (L / 2^32): the product's high part is reduced modulo 2^32 exactly, then the
// integer parts of both halves are added.
__device__ __forceinline__ unsigned int frac32_df(DF x, DF conv) {
    const DF y = df_mul(x, conv);
    const float k = rintf(__fmul_rn(y.h, 2.3283064365386963e-10f));
    const float t = __fsub_rn(y.h, __fmul_rn(k, 4294967296.0f));
    const float ti = rintf(t);
    const float r = __fadd_rn(__fsub_rn(t, ti), y.l);
    return (unsigned int)__float2int_rn(ti) + (unsigned int)__float2int_rn(r);
}

// ---------------------------------------------------------------------------------------------
// Thermostat chain on three warps.  The FP64 units of this GPU serve one sub-partition each at
// about 30 ns per dependent instruction, so the chain's time is its critical path.  The critical
// recurrence (steps 1.2 and 1.5 for p_eta[0..M-2]) runs on warp 0; warp 1 computes the step-1.4
// momentum scaling from p_eta[0] and carries the kinetic term; warp 2 owns p_eta[M-1] (steps 1.1
// and 1.6) and its exponential.  Values move through shared memory behind monotonically
// increasing sequence flags; every wait is bounded (on expiry the chain sets `timeout` and
// finishes with the values it has, so the kernel always terminates).
// Exact reuse: within one Suzuki-Yoshida stage the step-1.2 exponential of p_eta[j+1] equals the
// step-1.5 exponential of the previous substep (same argument), so it is not recomputed.  The
// step-1.5 exponentials are obtained from the step-1.2 ones by a fourth-order correction when the
// argument moved by less than 2^-10 (remainder below 1e-17), else evaluated afresh.
// ---------------------------------------------------------------------------------------------
struct NhExchange {
    double pe[kMaxChain];
    double eta[kMaxChain];
    double iQ[kMaxChain];
    double KE2, scale;
    double pe0, ke, pe_m2, etop;            // slots
    DF dpe0, dke, dpe_m2, detop;            // the same slots of the double-float chain
    // double-float hand-over slots: each half of the value in its own 64-bit word beside the
    // sequence number (see slot_post / slot_wait)
    unsigned long long q_pe0[2], q_ke[2], q_pe_m2[2], q_etop[2];
    volatile int f_pe0, f_ke, f_pe_m2, f_etop;
    int timeout;
    int polls;                              // wait limit (Params::wait_polls)
};

// Bounded wait for a flag of another warp of the block: spins on shared memory for the first
// 4096 polls (the partner is normally a few hundred cycles away), then backs off; gives up after
// the context's limit (Params::wait_polls, 2^22 by default) and records a timeout.
// Flag hand-over between warps of a block with release / acquire ordering at CTA scope: the
// posting lane's earlier shared-memory stores (the value) are visible to a waiter once it observes
// the flag, without a full block fence on either side.
__device__ __forceinline__ int ld_acquire_cta(volatile int* p) {
    int v;
    asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];"
                 : "=r"(v)
                 : "r"((unsigned)__cvta_generic_to_shared((void*)p))
                 : "memory");
    return v;
}
__device__ __forceinline__ void st_release_cta(volatile int* p, int v) {
    asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared((void*)p)), "r"(v)
                 : "memory");
}

__device__ __forceinline__ void nh_wait(volatile int* flag, int seq, int* timeout, int polls) {
    for(int it = 0; it < polls; it++) {
        if(ld_acquire_cta(flag) >= seq) return;
        if(it >= 4096) __nanosleep(32);
    }
    *timeout = 1;
}

// Hand-over of a double-float value without acquire / release: each float travels in its own
// aligned 64-bit word together with the sequence number, written by lane 0 with relaxed stores
// and polled with relaxed loads.  An aligned 64-bit access is single-copy atomic, so a reader that
// sees the expected sequence in both words has both halves of that post.  A producer never posts
// a slot again before its consumer has read it (each post waits on a value the consumer hands
// back after reading), so the expected sequence is the one present.  Bounded like nh_wait: after
// `polls` reads the wait records a timeout and returns what it has.
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"((unsigned)__cvta_generic_to_shared((void*)p)), "l"(v)
                 : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.cta.shared::cta.b64 %0, [%1];" : "=l"(v) : "r"((unsigned)__cvta_generic_to_shared((void*)p))
                 : "memory");
    return v;
}
__device__ __forceinline__ void slot_post(unsigned long long* q, DF v, int seq) {
    if((threadIdx.x & 31) == 0) {
        const unsigned long long tag = (unsigned long long)(unsigned)seq << 32;
        st_relaxed_u64(q, tag | __float_as_uint(v.h));
        st_relaxed_u64(q + 1, tag | __float_as_uint(v.l));
    }
}
__device__ __forceinline__ DF slot_wait(const unsigned long long* q, int seq, int* timeout, int polls) {
    unsigned long long a = 0, b = 0;
    for(int it = 0; it < polls; it++) {
        a = ld_relaxed_u64(q);
        b = ld_relaxed_u64(q + 1);
        if((int)(a >> 32) == seq && (int)(b >> 32) == seq) return DF{__uint_as_float((unsigned)a), __uint_as_float((unsigned)b)};
        if(it >= 4096) __nanosleep(32);
    }
    *timeout = 1;
    return DF{__uint_as_float((unsigned)a), __uint_as_float((unsigned)b)};
}

// Lane 0 posts; it is also the lane that stored the value being handed over.
__device__ __forceinline__ void nh_post(volatile int* flag, int seq) {
    if((threadIdx.x & 31) == 0) st_release_cta(flag, seq);
}

// e^x for |x| <= 2^-10 by its Taylor series to order 4 (remainder below 1e-17)
__device__ __forceinline__ double exp_tiny(double x) {
    double p = fma(x, 1.0 / 24.0, 1.0 / 6.0);
    p = fma(p, x, 0.5);
    p = fma(p, x, 1.0);
    return fma(p, x, 1.0);
}

// CMt::exp with branch tests on the bit pattern (x > 1) instead of FP64 comparisons
__device__ __forceinline__ double cmt_exp_bits(double x, bool fixed) {
    if(!fixed && __double_as_longlong(x) > 0x3ff0000000000000LL) return 2.71828 * x;
    return nh_exp(x);
}
// The same, not inlined: for branches that are rarely taken, whose FP64 instructions would
// otherwise be predicated into every pass
static __device__ __noinline__ double cmt_exp_call(double x, bool fixed) { return cmt_exp_bits(x, fixed); }

// One thermostat half-step on warps 0..2; M >= 2.  X holds the chain on entry and exit; the flags
// continue from `seq` (a counter shared by successive calls so flags only grow).  Returns the new
// counter value.
template<int MM>
__device__ inline int nh_chain_half_3w_t(NhExchange& X, double g, double kT, double dt, int M_rt, int nresp, int seq,
                                         bool fixed) {
    constexpr int CAP = MM > 0 ? MM : kMaxChain;   // register arrays when the length is known
    const int M = MM > 0 ? MM : M_rt;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double w0 = sy_w0(fixed);
    const double w[3] = {w0, 1.0 - 2.0 * w0, w0};
    // the two distinct Suzuki-Yoshida stage lengths w_mu dt / nresp, each FP64 division once per call
    const double DtS[2] = {w[0] * dt / double(nresp), w[1] * dt / double(nresp)};
    const double gkT = g * kT;
    const int top = M - 1;
    const int nsub = 3 * nresp;
    int* tmo = &X.timeout;
    const long long half_bits = 0x3fe0000000000000LL;       // 0.5
    const long long tiny_bits = 0x3f50000000000000LL;       // 2^-10
    if(warp == 0) {
        // ---------------- main: p_eta[0..M-2], steps 1.2 and 1.5 ----------------
        double pe[CAP], iQ[CAP], cprev[CAP], xprev[CAP];
        #pragma unroll
        for(int j = 0; j < M; j++) {
            pe[j] = X.pe[j];
            iQ[j] = X.iQ[j];
        }
        double KE2 = X.KE2;
        double eta_mine = (lane < top) ? X.eta[lane] : 0.0;
        if(!fixed && pe[0] > 15.0) pe[0] = 10.0;
        int s = 0;
        for(int mu = 0; mu < 3; mu++) {
            const double Dt = DtS[mu == 1 ? 1 : 0];
            const double d8 = -(Dt / 8.0), d4 = Dt / 4.0, d2 = Dt / 2.0;
            // per-stage coefficients: d4 G_j = pe[j-1]^2 A_j - B (j >= 1), d4 G_0 = KE2 d4 - B0,
            // exponent of c_j = pe[j+1] D_j, eta step d2 pe/Q = pe E
            double A[CAP], D[CAP];
#pragma unroll
            for(int j = 0; j < top; j++) {
                A[j] = (j > 0) ? d4 * iQ[j - 1] : 0.0;
                D[j] = d8 * iQ[j + 1];
            }
            const double B = d4 * kT, B0 = d4 * gkT;
            double E = 0.0;
#pragma unroll
            for(int j = 0; j < top; j++)
                if(j == lane) E = d2 * iQ[j];
            for(int it = 0; it < nresp; it++, s++) {
                double etop = 0.0;
                double c12[CAP], x12[CAP], t12[CAP];
                // 1.2
#pragma unroll
                for(int j = 0; j < top; j++) {
                    double c, x;
                    if(j == top - 1) {
                        nh_wait(&X.f_etop, seq + s + 1, tmo, X.polls);      // exponential of p_eta[M-1] (warp 2)
                        etop = X.etop;
                        c = etop;
                        x = 0.0;
                    } else if(it > 0) {
                        c = cprev[j];                       // same argument as step 1.5 before
                        x = xprev[j];
                    } else {
                        x = pe[j + 1] * D[j];
                        c = cmt_exp_call(x, fixed);
                    }
                    c12[j] = c;
                    x12[j] = x;
                    const double t = (j == 0) ? fma(KE2, d4, -B0) : fma(pe[j - 1] * pe[j - 1], A[j], -B);
                    t12[j] = t;
                    pe[j] = fma(pe[j], c, t) * c;
                    if(j == 0) {
                        if(lane == 0) X.pe0 = pe[0];
                        nh_post(&X.f_pe0, seq + s + 1);
                    }
                }
                // 1.3 (this warp's elements)
                {
                    double v = 0.0;
#pragma unroll
                    for(int j = 0; j < top; j++)
                        if(j == lane) v = pe[j];
                    if(lane < top) eta_mine = fma(v, E, eta_mine);
                }
                // 1.5
#pragma unroll
                for(int j = top - 1; j >= 0; j--) {
                    double c;
                    if(j == top - 1) {
                        c = etop;                           // p_eta[M-1] has not changed since 1.2
                    } else {
                        const double xn = pe[j + 1] * D[j];
                        const double dx = xn - x12[j];
                        if((__double_as_longlong(dx) & 0x7fffffffffffffffLL) <= tiny_bits &&
                           __double_as_longlong(xn) <= half_bits && __double_as_longlong(x12[j]) <= half_bits)
                            c = c12[j] * exp_tiny(dx);
                        else
                            c = cmt_exp_call(xn, fixed);
                        cprev[j] = c;
                        xprev[j] = xn;
                    }
                    double t;
                    if(j == 0) {
                        nh_wait(&X.f_ke, seq + s + 1, tmo, X.polls);    // kinetic term after step 1.4 (warp 1)
                        KE2 = X.ke;
                        t = fma(KE2, d4, -B0);
                    } else {
                        t = t12[j];   // p_eta[j-1] is as step 1.2 left it: the same driving term
                    }
                    pe[j] = fma(pe[j], c, t) * c;
                    if(j == top - 1) {
                        if(lane == 0) X.pe_m2 = pe[top - 1];
                        nh_post(&X.f_pe_m2, seq + s + 1);
                    }
                }
            }
        }
        __syncwarp();
        if(lane < top) {
            double v = 0.0;
#pragma unroll
            for(int j = 0; j < top; j++)
                if(j == lane) v = pe[j];
            X.pe[lane] = v;
            X.eta[lane] = eta_mine;
        }
    } else if(warp == 1) {
        // ---------------- warp 1: step 1.4, kinetic term, momentum scale ----------------
        const double iQ0 = X.iQ[0];
        double KE2 = X.KE2, scale = 1.0;
        int s = 0;
        for(int mu = 0; mu < 3; mu++) {
            const double d2 = DtS[mu == 1 ? 1 : 0] / 2.0;
            for(int it = 0; it < nresp; it++, s++) {
                nh_wait(&X.f_pe0, seq + s + 1, tmo, X.polls);
                const double c = cmt_exp_bits(-(d2 * (X.pe0 * iQ0)), fixed);
                scale *= c;
                KE2 *= c * c;
                if(lane == 0) X.ke = KE2;
                nh_post(&X.f_ke, seq + s + 1);
            }
        }
        if(lane == 0) {
            X.KE2 = KE2;
            X.scale = scale;
        }
    } else if(warp == 2) {
        // ---------------- warp 2: p_eta[M-1] (steps 1.1, 1.6), its exponential, eta[M-1] ----------------
        const double iQm = X.iQ[top - 1], iQt = X.iQ[top];
        double pt = X.pe[top];
        double eta_t = X.eta[top];
        double pm = X.pe[top - 1];
        if(!fixed && top - 1 == 0 && pm > 15.0) pm = 10.0;    // the guard on p_eta[0] (NHChain.cpp:61-65)
        int s = 0;
        double d4p = 0.0;   // the previous substep's Dt/4 (the same expression as its d4)
        for(int mu = 0; mu < 3; mu++) {
            const double Dt = DtS[mu == 1 ? 1 : 0];
            const double d8 = -(Dt / 8.0), d4 = Dt / 4.0, d2 = Dt / 2.0;
            for(int it = 0; it < nresp; it++, s++) {
                if(s > 0) {
                    // 1.6 of the previous substep, with that substep's Dt
                    nh_wait(&X.f_pe_m2, seq + s, tmo, X.polls);
                    pm = X.pe_m2;
                    pt += d4p * (pm * pm * iQm - kT);
                }
                pt += d4 * (pm * pm * iQm - kT);          // 1.1
                const double c = cmt_exp_bits(d8 * (pt * iQt), fixed);
                if(lane == 0) X.etop = c;
                nh_post(&X.f_etop, seq + s + 1);
                eta_t += d2 * (pt * iQt);                   // 1.3 for the top element
                d4p = d4;
            }
        }
        nh_wait(&X.f_pe_m2, seq + nsub, tmo, X.polls);             // 1.6 of the last substep
        pm = X.pe_m2;
        pt += d4p * (pm * pm * iQm - kT);
        if(lane == 0) {
            X.pe[top] = pt;
            X.eta[top] = eta_t;
        }
    }
    return seq + nsub;
}

// ---------------------------------------------------------------------------------------------
// The same three-warp chain in double-float arithmetic, for the mixed precision mode (published
// Suzuki-Yoshida weight, exponential, no clamp).  Each FP64 instruction of the chain's critical
// warp costs about 100 cycles on this GPU (measured with clock64: 3,340 cycles of arithmetic per
// substep for 33 FP64 instructions); a double-float multiply or add is a handful of dependent FP32
// operations of 4 cycles each.  Exponentials of small arguments take the x^4 tail of the Taylor
// series in FP32 (it is below 2e-8, so FP32's relative error leaves 3e-15 absolute) and the low
// orders in double-float.  State enters and leaves as FP64 in X; values between warps move as
// double-float pairs through the d* slots.
// ---------------------------------------------------------------------------------------------
// The chain uses the shorter double-float sum (one two-sum of the high parts, the low parts added
// in FP32): its error is 2^-47 of |a| + |b| rather than of |a + b|, which for the chain's momenta,
// whose scale is set by their largest terms, is as good and 4 dependent operations shorter.
__device__ __forceinline__ DF df_addq(DF a, DF b) {
    const DF s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
// a b + c without renormalising the product first: the exact product p + e (e by fma), the cross
// terms and c's low part summed in FP32 beside the exact two_sum of p and c's high part; about
// 20 cycles shorter on a dependency chain than df_addq(df_mul(a, b), c), with the same error bound
// (about 2^-46 of |ab| + |c|)
__device__ __forceinline__ DF df_fma(DF a, DF b, DF c) {
    const float p = __fmul_rn(a.h, b.h);
    const float e = __fmaf_rn(a.h, b.h, -p);
    const float cr = __fmaf_rn(a.l, b.h, __fmul_rn(a.h, b.l));
    const DF s = two_sum(p, c.h);
    return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(__fadd_rn(e, cr), c.l)));
}
__device__ __forceinline__ DF df_scale(DF a, float pow2) { return {a.h * pow2, a.l * pow2}; }   // exact

// e^x for |x| > 1/2 through FP64, not inlined (see nh_exp): warps reach it only when a lane needs it
static __device__ __noinline__ DF df_exp_wide(DF x) { return df_of(nh_exp(df_val(x))); }

// e^x, |x| <= 2^-5, in double-float: 1 + x + x^2/2 + x^3/6 in double-float, the rest in FP32
__device__ __forceinline__ DF df_exp_small(DF x) {
    const float xf = x.h;
    float t = fmaf(xf, 1.0f / 40320.0f, 1.0f / 5040.0f);
    t = fmaf(t, xf, 1.0f / 720.0f);
    t = fmaf(t, xf, 1.0f / 120.0f);
    t = fmaf(t, xf, 1.0f / 24.0f);
    const float x2f = xf * xf;
    const float tail = t * (x2f * x2f);                                  // x^4/24 + ... + x^8/8!
    const DF sixth{0x1.555556p-3f, -0x1.555556p-28f};                     // 1/6
    const DF a = df_addq(df_mul(x, sixth), DF{0.5f, 0.0f});               // 1/2 + x/6
    const DF b = df_addq(df_mul(df_mul(x, x), a), DF{tail, 0.0f});         // x^2/2 + x^3/6 + tail
    return df_addq(df_addq(DF{1.0f, 0.0f}, x), b);
}

// e^x for the double-float chain.  |x| <= 2^-5 directly; |x| <= 1/2 as (e^(x/2^k))^(2^k) with k = 2
// or 4 exact halvings and k double-float squarings (relative error about 2^k times that of one
// product, 2^-46 for |x| <= 1/8); larger arguments through FP64.  The top chain element's argument
// Dt/8 p_eta/Q is often above 2^-5, where the FP64 route cost about 24 FP64 instructions per call
// on the chain's critical path.
__device__ __forceinline__ DF df_exp_chain(DF x) {
    const float ax = fabsf(x.h);
    if(ax <= 0.03125f) return df_exp_small(x);
    if(ax <= 0.5f) {
        const bool two = ax <= 0.125f;
        DF e = df_exp_small(df_scale(x, two ? 0.25f : 0.0625f));
        e = df_mul(e, e);
        e = df_mul(e, e);
        if(!two) {
            e = df_mul(e, e);
            e = df_mul(e, e);
        }
        return e;
    }
    return df_exp_wide(x);
}

// e^x, |x| <= 2^-10: 1 + x + x^2/2 in double-float, x^3/6 + x^4/24 (below 2e-10) in FP32
__device__ __forceinline__ DF df_exp_tiny(DF x) {
    const float xf = x.h;
    const float tail = (xf * xf) * (xf * fmaf(xf, 1.0f / 24.0f, 1.0f / 6.0f));
    const DF x2h = df_mul(x, DF{0.5f * x.h, 0.5f * x.l});
    return df_addq(df_addq(DF{1.0f, 0.0f}, x), df_addq(x2h, DF{tail, 0.0f}));
}

template<int MM>
__device__ inline int nh_chain_half_3w_df(NhExchange& X, double g, double kT, const double* stage, int M_rt, int nresp,
                                          int seq) {
    constexpr int CAP = MM > 0 ? MM : kMaxChain;
    const int M = MM > 0 ? MM : M_rt;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned full = 0xffffffffu;
    const int top = M - 1;
    const int nsub = 3 * nresp;
    int* tmo = &X.timeout;
    const float tiny = 0.0009765625f;   // 2^-10
    // FP64 -> double-float conversions run one value per lane: an FP64 instruction costs the
    // same for one lane as for 32 on this GPU, so a warp converts its inputs in one pass and
    // hands them out by shuffles.  Lanes 0..15 take one table, lanes 16..31 another.
    auto from = [&](const DF& mine, int l) { return DF{__shfl_sync(full, mine.h, l), __shfl_sync(full, mine.l, l)}; };
    if(warp == 0) {
        // ---------------- main: p_eta[0..M-2], steps 1.2 and 1.5 ----------------
        // every per-stage constant is then a double-float product (the Suzuki-Yoshida stages have
        // two distinct lengths, stage[0] and stage[1])
        DF pe[CAP], iQ[CAP], cprev[CAP], xprev[CAP];
        const int l16 = lane & 15;
        double v1 = (lane < 16) ? X.pe[l16 < M ? l16 : 0] : X.iQ[l16 < M ? l16 : 0];
        double v2 = (lane == 0) ? X.KE2 : (lane == 1) ? kT : (lane == 2) ? g * kT : (lane == 3) ? stage[0] : stage[1];
        const DF c1 = df_of(v1), c2 = df_of(v2);
#pragma unroll
        for(int j = 0; j < M; j++) {
            pe[j] = from(c1, j);
            iQ[j] = from(c1, 16 + j);
        }
        DF KE2 = from(c2, 0);
        DF eta_mine = df_of((lane < top) ? X.eta[lane] : 0.0);
        const DF kTD = from(c2, 1), gkTD = from(c2, 2);
        const DF DtW[2] = {from(c2, 3), from(c2, 4)};
        DF iQl{0.0f, 0.0f};
#pragma unroll
        for(int j = 0; j < top; j++)
            if(j == lane) iQl = iQ[j];
        int s = 0;
        for(int mu = 0; mu < 3; mu++) {
            const DF Dt = DtW[mu == 1 ? 1 : 0];
            const DF d8 = df_scale(Dt, -0.125f), d4D = df_scale(Dt, 0.25f), d2 = df_scale(Dt, 0.5f);
            DF A[CAP], D[CAP];
#pragma unroll
            for(int j = 0; j < top; j++) {
                A[j] = (j > 0) ? df_mul(d4D, iQ[j - 1]) : DF{0.0f, 0.0f};
                D[j] = df_mul(d8, iQ[j + 1]);
            }
            const DF nB = df_neg(df_mul(d4D, kTD)), nB0 = df_neg(df_mul(d4D, gkTD));
            const DF E = df_mul(d2, iQl);
            for(int it = 0; it < nresp; it++, s++) {
                DF etop{1.0f, 0.0f};
                DF c12[CAP], x12[CAP], t12[CAP];
                // 1.2
#pragma unroll
                for(int j = 0; j < top; j++) {
                    DF c, x;
                    if(j == top - 1) {
                        etop = slot_wait(X.q_etop, seq + s + 1, tmo, X.polls);   // exponential of p_eta[M-1] (warp 2)
                        c = etop;
                        x = DF{0.0f, 0.0f};
                    } else if(it > 0) {
                        c = cprev[j];
                        x = xprev[j];
                    } else {
                        x = df_mul(pe[j + 1], D[j]);
                        c = df_exp_chain(x);
                    }
                    c12[j] = c;
                    x12[j] = x;
                    const DF t = (j == 0) ? df_fma(KE2, d4D, nB0) : df_fma(df_mul(pe[j - 1], pe[j - 1]), A[j], nB);
                    t12[j] = t;
                    pe[j] = df_mul(df_fma(pe[j], c, t), c);
                    if(j == 0) slot_post(X.q_pe0, pe[0], seq + s + 1);
                }
                // 1.3 (this warp's elements)
                {
                    DF v{0.0f, 0.0f};
#pragma unroll
                    for(int j = 0; j < top; j++)
                        if(j == lane) v = pe[j];
                    if(lane < top) eta_mine = df_fma(v, E, eta_mine);
                }
                // 1.5
#pragma unroll
                for(int j = top - 1; j >= 0; j--) {
                    DF c;
                    if(j == top - 1) {
                        c = etop;
                    } else {
                        const DF xn = df_mul(pe[j + 1], D[j]);
                        const DF dx = df_addq(xn, df_neg(x12[j]));
                        if(fabsf(dx.h) <= tiny && xn.h <= 0.5f && x12[j].h <= 0.5f)
                            c = df_mul(c12[j], df_exp_tiny(dx));
                        else
                            c = df_exp_chain(xn);
                        cprev[j] = c;
                        xprev[j] = xn;
                    }
                    DF t;
                    if(j == 0) {
                        KE2 = slot_wait(X.q_ke, seq + s + 1, tmo, X.polls);   // kinetic term after step 1.4 (warp 1)
                        t = df_fma(KE2, d4D, nB0);
                    } else {
                        t = t12[j];
                    }
                    pe[j] = df_mul(df_fma(pe[j], c, t), c);
                    if(j == top - 1) slot_post(X.q_pe_m2, pe[top - 1], seq + s + 1);
                }
            }
        }
        __syncwarp();
        {
            // lanes 0..top-1 return p_eta, lanes 16..16+top-1 eta, in one conversion pass
            const int l16 = lane & 15;
            DF v{0.0f, 0.0f};
#pragma unroll
            for(int j = 0; j < top; j++)
                if(j == l16) v = pe[j];
            const DF e = from(eta_mine, l16);
            const double o = df_val(lane < 16 ? v : e);
            if(l16 < top) {
                if(lane < 16) X.pe[l16] = o;
                else X.eta[l16] = o;
            }
        }
    } else if(warp == 1) {
        // ---------------- warp 1: step 1.4, kinetic term, momentum scale ----------------
        const double v = (lane == 0) ? X.iQ[0] : (lane == 1) ? X.KE2 : (lane == 2) ? stage[0] : stage[1];
        const DF cv = df_of(v);
        const DF iQ0 = from(cv, 0);
        DF KE2 = from(cv, 1), scale{1.0f, 0.0f};
        const DF D1W[2] = {df_neg(df_mul(from(cv, 2), df_scale(iQ0, 0.5f))), df_neg(df_mul(from(cv, 3), df_scale(iQ0, 0.5f)))};
        int s = 0;
        for(int mu = 0; mu < 3; mu++) {
            const DF D1 = D1W[mu == 1 ? 1 : 0];
            for(int it = 0; it < nresp; it++, s++) {
                const DF p0 = slot_wait(X.q_pe0, seq + s + 1, tmo, X.polls);
                const DF c = df_exp_chain(df_mul(p0, D1));
                scale = df_mul(scale, c);
                KE2 = df_mul(KE2, df_mul(c, c));
                slot_post(X.q_ke, KE2, seq + s + 1);
            }
        }
        const DF out = (lane == 0) ? KE2 : scale;
        const double o = df_val(out);   // both in one pass
        if(lane == 0) X.KE2 = o;
        if(lane == 1) X.scale = o;
    } else if(warp == 2) {
        // ---------------- warp 2: p_eta[M-1] (steps 1.1, 1.6), its exponential, eta[M-1] ----------------
        const double v = (lane == 0) ? X.iQ[top] : (lane == 1) ? X.iQ[top - 1] : (lane == 2) ? -kT
                         : (lane == 3) ? stage[0] : (lane == 4) ? stage[1] : (lane == 5) ? X.pe[top]
                         : (lane == 6) ? X.eta[top] : X.pe[top - 1];
        const DF cv = df_of(v);
        const DF iQt = from(cv, 0);
        const DF iQm = from(cv, 1), nkT = from(cv, 2);
        const DF DtW[2] = {from(cv, 3), from(cv, 4)};
        DF pt = from(cv, 5);
        DF eta_t = from(cv, 6);
        DF pm = from(cv, 7);
        DF d4prev{0.0f, 0.0f};
        int s = 0;
        for(int mu = 0; mu < 3; mu++) {
            const DF Dt = DtW[mu == 1 ? 1 : 0];
            const DF d4 = df_scale(Dt, 0.25f), Dtop = df_mul(df_scale(Dt, -0.125f), iQt), Etop = df_mul(df_scale(Dt, 0.5f), iQt);
            for(int it = 0; it < nresp; it++, s++) {
                if(s > 0) {
                    // 1.6 of the previous substep, with that substep's Dt
                    pm = slot_wait(X.q_pe_m2, seq + s, tmo, X.polls);
                    pt = df_fma(d4prev, df_fma(df_mul(pm, pm), iQm, nkT), pt);
                }
                pt = df_fma(d4, df_fma(df_mul(pm, pm), iQm, nkT), pt);         // 1.1
                const DF c = df_exp_chain(df_mul(pt, Dtop));
                slot_post(X.q_etop, c, seq + s + 1);
                eta_t = df_fma(pt, Etop, eta_t);                               // 1.3 for the top element
                d4prev = d4;
            }
        }
        pm = slot_wait(X.q_pe_m2, seq + nsub, tmo, X.polls);      // 1.6 of the last substep
        pt = df_fma(d4prev, df_fma(df_mul(pm, pm), iQm, nkT), pt);
        const double o = df_val((lane == 0) ? pt : eta_t);   // both in one pass
        if(lane == 0) X.pe[top] = o;
        if(lane == 1) X.eta[top] = o;
    }
    return seq + nsub;
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
// The same election among the `nblocks` blocks that share `counter` (one replica of a batch).
__device__ inline bool last_block_of(unsigned int* counter, unsigned int nblocks) {
    __shared__ bool is_last_of;
    __threadfence();
    __syncthreads();
    if(threadIdx.x == 0) {
        unsigned int prev = atomicAdd(counter, 1u);
        is_last_of = (prev == nblocks - 1);
    }
    __syncthreads();
    if(is_last_of) __threadfence();
    return is_last_of;
}

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

// One chain half-step on warps 0..2, inlined into each kernel that runs one.  DFLOAT selects the
// double-float family (mixed mode) or the FP64 family at compile time, so a kernel carries only
// the family it uses: register arrays for the default chain length 4, the runtime-length form
// for any other.
template<bool DFLOAT>
__device__ __forceinline__ int nh_chain_half_3w(NhExchange& X, double g, double kT, double dt, int M, int nresp, int seq,
                                                bool fixed, const double* stage) {
    if constexpr(DFLOAT) {
        if(M == 4) return nh_chain_half_3w_df<4>(X, g, kT, stage, M, nresp, seq);
        return nh_chain_half_3w_df<0>(X, g, kT, stage, M, nresp, seq);
    } else {
        if(M == 4) return nh_chain_half_3w_t<4>(X, g, kT, dt, M, nresp, seq, fixed);
        return nh_chain_half_3w_t<0>(X, g, kT, dt, M, nresp, seq, fixed);
    }
}

__device__ __forceinline__ void bar96() { asm volatile("bar.sync 1, 96;" ::: "memory"); }

// Chain half-steps for the end of a step (second half of this step, then first half of the
// next: MDLoop.cpp:129-132) or for the prologue of a run (first half only), run by warps 0..2 of
// one block (threadIdx.x < 96).  th_saved receives the chain after the second half-step (the
// state the reference holds between steps).  Returns (via *c2, *c1) the scales of the driven
// momentum, KE2 after the second half-step and, in *KE_full, after both.  The particle chain has
// g = 3N (CFctT, MDLoop.cpp:29-60); the barostat's chain g = 1 with KE2 = p_eps^2/W (CFctP,
// MDLoop.cpp:62-83).
template<bool DFLOAT>
__device__ inline void thermostat_chain(const Params& P, StepScalars* sc, ThermoDev* th, ThermoDev* th_saved,
                                        double& KE2, bool second_half, double* c2_out, double* c1_out,
                                        double g, int M, int nresp, double* KE_full) {
    __shared__ NhExchange X;
    const int tid = threadIdx.x;
    const bool fixed = P.precision != MTG_PREC_REFERENCE;
    double c2 = 1.0, c1 = 1.0;
    double KEf = KE2;
    if(M >= 2) {
        if(tid < kMaxChain) {
            X.pe[tid] = th->peta[tid];
            X.eta[tid] = th->eta[tid];
            X.iQ[tid] = th->iQ[tid];
        }
        if(tid == 0) {
            X.KE2 = KE2;
            X.scale = 1.0;
            X.f_pe0 = X.f_ke = X.f_pe_m2 = X.f_etop = 0;
            X.q_pe0[0] = X.q_pe0[1] = X.q_ke[0] = X.q_ke[1] = 0ULL;
            X.q_pe_m2[0] = X.q_pe_m2[1] = X.q_etop[0] = X.q_etop[1] = 0ULL;
            X.timeout = 0;
            X.polls = P.wait_polls;
        }
        bar96();
        int seq = 0;
        if(second_half) {
            seq = nh_chain_half_3w<DFLOAT>(X, g, P.kT, P.dt, M, nresp, seq, fixed, P.chain_stage);
            bar96();
            c2 = X.scale;
            if(tid < M) {
                th_saved->peta[tid] = X.pe[tid];
                th_saved->eta[tid] = X.eta[tid];
            }
            bar96();
            if(tid == 0) X.scale = 1.0;
            bar96();
        } else {
            if(tid < M) {
                th_saved->peta[tid] = X.pe[tid];
                th_saved->eta[tid] = X.eta[tid];
            }
        }
        const double KE_after2 = X.KE2;
        bar96();
        seq = nh_chain_half_3w<DFLOAT>(X, g, P.kT, P.dt, M, nresp, seq, fixed, P.chain_stage);
        bar96();
        c1 = X.scale;
        KEf = X.KE2;
        KE2 = KE_after2;
        if(tid < M) {
            th->peta[tid] = X.pe[tid];
            th->eta[tid] = X.eta[tid];
        }
        if(tid == 0 && X.timeout) sc->timeout = 1;
        bar96();   // X is reused by the next chain of this block
    } else if(M == 1 && tid < 32) {
        if(second_half) {
            c2 = nh_chain_half(*th, KE2, g, P.kT, P.dt, M, nresp, fixed);
            __threadfence_block();
            if(tid == 0) {
                th_saved->eta[0] = th->eta[0];
                th_saved->peta[0] = th->peta[0];
            }
        } else if(tid == 0) {
            th_saved->eta[0] = th->eta[0];
            th_saved->peta[0] = th->peta[0];
        }
        __syncwarp();
        double KEn = KE2;
        c1 = nh_chain_half(*th, KEn, g, P.kT, P.dt, M, nresp, fixed);
        KEf = KEn;
    }
    *c2_out = c2;
    *c1_out = c1;
    if(KE_full) *KE_full = KEf;
}

template<bool DFLOAT>
__device__ inline void thermostat(const Params& P, StepScalars* sc, ThermoDev* th, ThermoDev* th_saved,
                                  double& KE2, bool second_half, double* c2_out, double* c1_out) {
    thermostat_chain<DFLOAT>(P, sc, th, th_saved, KE2, second_half, c2_out, c1_out, double(3 * P.n), P.M, P.nresp, nullptr);
}

// End-of-step scalar work of the last block, run by its warps 0..2 (threadIdx.x < 96): the
// thermostat half-steps and the output scalars.
template<bool DFLOAT>
__device__ inline void end_of_step(const Params& P, StepScalars* sc, ThermoDev* th, ThermoDev* th_saved,
                                   double KE2, double U, double vir, bool output, double* rec) {
    double c2 = 1.0, c1 = 1.0;
    if(P.ensemble == MTG_NVT || P.ensemble == MTG_NPT) thermostat<DFLOAT>(P, sc, th, th_saved, KE2, true, &c2, &c1);
    if(threadIdx.x == 0) {
        if(!isfinite(KE2) || !isfinite(c2 * c1)) sc->nonfinite = 1;
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

// CMt::sinhXoverX (Math.cpp:40-54): the first six terms of the Taylor series of sinh(x)/x.
__device__ inline double sinhx_over_x(double x) {
    const double a[6] = {1.0, 1.0 / 6.0, 1.0 / 120.0, 1.0 / 5040.0, 1.0 / 362880.0, 1.0 / 39916800.0};
    double sum = 0.0, xn = 1.0;
#pragma unroll
    for(int k = 0; k < 6; k++) {
        sum += a[k] * xn;
        xn *= (x * x);
    }
    return sum;
}

// NPT scalar work (MDLoop.cpp:128-133 with VelVerlet.cpp:57-71), run by warps 0..2 of the last
// block of a step (second_half) or of a run's prologue.  In order:
//   3.6  p_eps += dt/2 G_eps(p after 3.5, F, unwrapped r)           (end of a step only)
//   NH_T second half + next first half; NH_P second half + next first half (the chains act on
//        disjoint variables, so running NH_T's pair before NH_P's equals the reference order)
//   output record of the completed step (V = V0 exp(3 eps))
//   3.1  p_eps += dt/2 G_eps(p after NH_T, F, wrapped r) of the next step
//   prop_p / prop_r coefficients, 3.4 eps += dt p_eps / W, and the next box getSimBox().
// G_eps = (1 + 1/N) sum p^2/m + sum F.r - 3 P V (VelVerlet.cpp:160-174).
// The production modes pass the pair virial (sum over pairs of r_ij . F_ij plus the bonded terms'
// virial) as both virials, use the exponential itself for the coefficients (and the chains'
// published Suzuki-Yoshida weights, as their NVT does), run the particle chain in double-float
// in the mixed mode (DFLOAT), and derive the box fields the production kernels read.
template<bool DFLOAT>
__device__ inline void npt_scalars(const Params& P, const DevSys& d, double KE2, double vir_unw, double vir_wr,
                                   double U, bool second_half, bool output) {
    __shared__ double sh_kep;
    const int tid = threadIdx.x;
    BaroDev* b = d.baro;
    const double dt = P.dt;
    const bool prod = P.precision != MTG_PREC_REFERENCE;
    const double alpha = (1.0 + 1.0 / double(P.n));
    if(second_half && tid == 0) {
        const double V = P.V0 * exp(3.0 * b->eps);
        b->p_eps += ((dt / 2.0) * (alpha * KE2 + vir_unw - 3.0 * P.Pext * V));
    }
    bar96();
    double c2 = 1.0, c1 = 1.0, KEf = KE2;
    thermostat_chain<DFLOAT>(P, d.sc, d.th, d.th_saved, KE2, second_half, &c2, &c1, double(3 * P.n), P.M, P.nresp, &KEf);
    bar96();
    if(tid == 0) sh_kep = b->p_eps * b->p_eps / P.W;
    bar96();
    double KEp = sh_kep, c2p = 1.0, c1p = 1.0;
    thermostat_chain<false>(P, d.sc, d.thp, d.thp_saved, KEp, second_half, &c2p, &c1p, 1.0, P.MP, P.nrespP, nullptr);
    bar96();
    if(tid == 0) {
        StepScalars* sc = d.sc;
        double pe = b->p_eps * c2p;            // after NH_P's second half: the completed step
        b->p_eps_saved = pe;
        b->eps_saved = b->eps;
        for(int a = 0; a < 3; a++) b->L_saved[a] = b->L[a];
        sc->c2 = c2;
        sc->S = c2 * c1;
        sc->KE2 = KE2;
        double V = P.V0 * exp(3.0 * b->eps);
        if(output) {
            d.rec[0] = U;
            d.rec[1] = 0.5 * KE2;
            d.rec[2] = KE2 / (3.0 * double(P.n));
            d.rec[3] = (1.0 / (3.0 * V)) * (KE2 + vir_wr);
            d.rec[4] = V;
            sc->U = U;
            sc->virial = vir_wr;
        }
        pe *= c1p;
        pe += ((dt / 2.0) * (alpha * KEf + vir_wr - 3.0 * P.Pext * V));   // 3.1
        b->p_eps = pe;
        const double u = pe / P.W;
        double parm = alpha * u * dt / 4.0;
        double co = prod ? exp(-parm) : cmt_exp(-parm);
        b->ap = co * co;
        b->bp = (dt / 2.0) * co * sinhx_over_x(parm);
        parm = u * dt / 2.0;
        co = prod ? exp(parm) : cmt_exp(parm);
        b->ar = co * co;
        b->br = dt * (sinhx_over_x(parm) * co);
        b->eps += (dt * pe / P.W);                                          // 3.4
        const double Vmax = P.box[0] * P.box[1] * P.box[2];
        double ec = (P.V0 * exp(3.0 * b->eps)) / Vmax;
        ec = pow(ec, 1.0 / 3.0);
        for(int a = 0; a < 3; a++) {
            b->L[a] = ec * P.box[a];
            b->Lf[a] = (float)b->L[a];
        }
        if(prod && !baro_box_fields(P, *b)) sc->boxerr = 1;
        if(!isfinite(KE2) || !isfinite(pe) || !isfinite(c2 * c1)) sc->nonfinite = 1;
    }
}

// Minimum image by rounding (production kernels).
__device__ __forceinline__ float minimg_f(float d, float L, float invL) { return d - L * rintf(d * invL); }
__device__ __forceinline__ double minimg_d(double d, double L, double invL) { return d - L * rint(d * invL); }

}  // namespace mtg
