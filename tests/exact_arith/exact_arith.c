/* CPU check of the exact-arithmetic steps of the reference-precision all-pairs Coulomb kernel
 * (moltwister_gb300/csrc/ref_kernels.cu: dist_to_float, quot_ff, image_sep), restated here in C
 * with the same FP32 and integer operations, against the FP64 operations they replace:
 *   R = (float)sqrt(x*x + y*y + z*z)          (FunctorCalcForce.cpp:258-278: float R of the FP64 norm)
 *   q = (double)K / (double)R3                (K, R3 floats)
 *   shift = |c - v| > w/2                     (Utilities/3DVector.cpp:133-165)
 * on seeded random inputs of the Coulomb loop's ranges and on inputs built to sit at or next to
 * the rounding boundaries.  Prints the mismatch counts and the share of inputs that took the
 * FP64 fallback; exits 1 on any mismatch.  Test infrastructure: build with -ffp-contract=off. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;
static double d_of(long long b) { double d; memcpy(&d, &b, 8); return d; }
static long long b_of(double d) { long long b; memcpy(&b, &d, 8); return b; }
static float f_of(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t u_of(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }
static long slow_r, slow_q, slow_i;

static float dist_fp64(double x, double y, double z) { slow_r++; return (float)sqrt(x * x + y * y + z * z); }
static double quot_fp64(float K, float R) { slow_q++; return (double)K / (double)R; }

static int split_df(double x, float* hi, float* lo) {
    long long b = b_of(x);
    int ex = (int)((b >> 52) & 0x7ff);
    if((b & 0x7fffffffffffffffLL) == 0) { *hi = *lo = 0.0f; return 1; }
    if(ex < 1023 - 60 || ex > 1023 + 60) return 0;
    uint32_t sgn = (uint32_t)((unsigned long long)b >> 63) << 31;
    *hi = f_of(sgn | ((uint32_t)(ex - 1023 + 127) << 23) | (uint32_t)((b >> 29) & 0x7fffff));
    float l = (float)(uint32_t)(b & 0x1fffffff) * f_of((uint32_t)(ex - 1075 + 127) << 23);
    *lo = f_of(u_of(l) | sgn);
    return 1;
}
static void two_sum(float a, float b, float* s, float* t) {
    float ss = a + b, bb = ss - a;
    *s = ss;
    *t = (a - (ss - bb)) + (b - bb);
}
static float dist_to_float(double x, double y, double z) {
    float xh, xl, yh, yl, zh, zl;
    if(!split_df(x, &xh, &xl) || !split_df(y, &yh, &yl) || !split_df(z, &zh, &zl)) return dist_fp64(x, y, z);
    float px = xh * xh, ex = fmaf(xh, xh, -px);
    float py = yh * yh, ey = fmaf(yh, yh, -py);
    float pz = zh * zh, ez = fmaf(zh, zh, -pz);
    float s1, t1, s2, t2;
    two_sum(px, py, &s1, &t1);
    two_sum(s1, pz, &s2, &t2);
    float cross = (xh * xl + yh * yl) + zh * zl;
    float low = (xl * xl + yl * yl) + zl * zl;
    float c = (((t1 + t2) + ((ex + ey) + ez)) + 2.0f * cross) + low;
    float Sh = s2 + c, Sl = c - (Sh - s2);
    if(!(Sh >= 0x1p-100f)) {
        if(x == 0.0 && y == 0.0 && z == 0.0) return 0.0f;
        return dist_fp64(x, y, z);
    }
    const float lo = 1.0f - 0x1p-12f, hi = 1.0f + 0x1p-12f;
    float a = sqrtf(Sh);
    float Er = fmaf(-a, a, Sh) + Sl;
    uint32_t ab = u_of(a);
    float U = f_of((ab & 0x7f800000u) - (23u << 23));
    float D = ((ab & 0x7fffffu) == 0) ? 0.5f * U : U;
    float tu = a * U, td = a * D;
    if(Er < tu * lo && Er > -td * lo) return a;
    if(Er > tu * hi || Er < -td * hi) {
        int up = Er > 0.0f;
        float a1 = f_of(up ? ab + 1u : ab - 1u);
        uint32_t b1 = u_of(a1);
        float U1 = f_of((b1 & 0x7f800000u) - (23u << 23));
        float D1 = ((b1 & 0x7fffffu) == 0) ? 0.5f * U1 : U1;
        float Er1 = up ? Er - 2.0f * tu : Er + 2.0f * td;
        if(Er1 < (a1 * U1) * lo && Er1 > -(a1 * D1) * lo) return a1;
    }
    return dist_fp64(x, y, z);
}
static double quot_ff(float K, float R) {
    uint32_t kb = u_of(K), rb = u_of(R);
    int ke = (int)((kb >> 23) & 0xff), re = (int)((rb >> 23) & 0xff);
    if(ke < 127 - 60 || ke > 127 + 60 || re < 127 - 60 || re > 127 + 60 || ke - re < -40 || ke - re > 40 || (rb >> 31))
        return quot_fp64(K, R);
    float Ka = f_of(kb & 0x7fffffffu);
    float q1 = Ka / R;
    float r1 = fmaf(-R, q1, Ka);
    float q2 = r1 / R;
    float r2 = fmaf(-R, q2, r1);
    float q3 = r2 * (1.0f / R);
    uint32_t b1 = u_of(q1);
    int e1 = (int)(b1 >> 23);
    u128 V = (u128)((b1 & 0x7fffffu) | 0x800000u) << 72;
    for(int i = 0; i < 2; i++) {
        uint32_t bf = u_of(i == 0 ? q2 : q3);
        if((bf & 0x7fffffffu) == 0) continue;
        int ef = (int)((bf >> 23) & 0xff);
        u128 M = (u128)((bf & 0x7fffffu) | 0x800000u);
        int sh = ef - e1 + 72;
        u128 c = sh >= 0 ? (M << sh) : (sh > -64 ? (M >> (-sh)) : (u128)0);
        if(bf >> 31) V -= c; else V += c;
    }
    if(!(V >> 94)) return quot_fp64(K, R);
    int msb = (V >> 95) ? 95 : 94;
    int drop = msb - 52;
    unsigned long long sig = (unsigned long long)(V >> drop);
    u128 rem = V & (((u128)1 << drop) - 1), half = (u128)1 << (drop - 1);
    if(rem + 16 >= half && rem <= half + 16) return quot_fp64(K, R);
    if(rem > half) sig++;
    unsigned long long bits = ((unsigned long long)(msb + e1 - 222 + 1023) << 52) + sig - (1ULL << 52);
    return d_of((long long)(bits | ((unsigned long long)(kb >> 31) << 63)));
}
static float trunc_f(double x) {
    long long b = b_of(x);
    int ex = (int)((b >> 52) & 0x7ff) - 1023 + 127;
    uint32_t sgn = (uint32_t)((unsigned long long)b >> 63) << 31;
    if(ex <= 0) return f_of(sgn);
    if(ex >= 255) return f_of(sgn | 0x7fc00000u);
    return f_of(sgn | ((uint32_t)ex << 23) | (uint32_t)((b >> 29) & 0x7fffff));
}
/* 1: shift, 0: none (the FP32 decision with its margin, else the FP64 test) */
static int image_shift(double c, double v, double w) {
    float cf = trunc_f(c), vf = trunc_f(v), hwf = (float)(w / 2.0);
    float d = fabsf(cf - vf);
    float m = 0x1p-20f * ((fabsf(cf) + fabsf(vf)) + hwf);
    if(d > hwf + m) return 1;
    if(d < hwf - m) return 0;
    slow_i++;
    return fabs(c - v) > w / 2.0;
}

static uint64_t st = 0x9E3779B97F4A7C15ULL;
static uint64_t rnd(void) { st ^= st << 13; st ^= st >> 7; st ^= st << 17; return st; }
static double urand(void) { return (double)(rnd() >> 11) * (1.0 / 9007199254740992.0); }

int main(int argc, char** argv) {
    long N = argc > 1 ? atol(argv[1]) : 2000000;
    long bad_r = 0, bad_q = 0, bad_i = 0;
    for(long t = 0; t < N; t++) {
        double x, y, z;
        int cls = (int)(t % 4);
        if(cls == 0) { x = (urand() - 0.5) * 90.0; y = (urand() - 0.5) * 90.0; z = (urand() - 0.5) * 90.0; }
        else if(cls == 1) { x = (urand() - 0.5) * 3.0; y = (urand() - 0.5) * 1e-3; z = (urand() - 0.5) * 30.0; }
        else if(cls == 2) { x = (double)(int)(urand() * 20) * 0.5; y = (double)(int)(urand() * 10) * 0.25; z = 0.0; }
        else {
            /* sums of squares at and next to the squares of float midpoints */
            float a = (float)(urand() * 40.0 + 0.5);
            double m = (double)a + ldexp(1.0, ilogbf(a) - 24);
            x = 0.0; y = 0.0;
            z = d_of(b_of(m) + (long long)(rnd() % 9) - 4);
        }
        float R = dist_to_float(x, y, z), Rw = (float)sqrt(x * x + y * y + z * z);
        if(u_of(R) != u_of(Rw)) { if(bad_r < 5) printf("R mismatch %a %a %a: %a vs %a\n", x, y, z, R, Rw); bad_r++; }
        float K = (float)((urand() - 0.5) * 2000.0);
        float R3 = Rw * Rw * Rw;
        if(t % 5 == 0) R3 = f_of(((uint32_t)rnd() & 0x3fffffffu) | 0x20000000u);
        if(t % 7 == 0) K = f_of(((uint32_t)rnd() & 0x3fffffffu) | 0x20000000u | (uint32_t)(rnd() & 1) << 31);
        if(K != 0.0f && R3 != 0.0f && !isnan(K) && !isnan(R3)) {
            double q = quot_ff(K, R3), qw = (double)K / (double)R3;
            if(b_of(q) != b_of(qw)) { if(bad_q < 5) printf("q mismatch %a / %a: %a vs %a\n", K, R3, q, qw); bad_q++; }
        }
        /* minimum image: positions in [-L/2, L/2], separations at and around L/2 */
        double L = 20.0 + urand() * 60.0;
        double w = (double)(float)L / 2.0 - (-(double)(float)L / 2.0);
        double c = (urand() - 0.5) * L, v;
        if(t % 3 == 0) v = c - w / 2.0 + (double)((long long)(rnd() % 17) - 8) * ldexp(1.0, ilogb(w) - 52);
        else if(t % 3 == 1) v = c - (w / 2.0) * (1.0 + ((rnd() & 1) ? 1.0 : -1.0) * ldexp(1.0, -(int)(14 + rnd() % 14)));
        else v = (urand() - 0.5) * L;
        if(image_shift(c, v, w) != (fabs(c - v) > w / 2.0)) bad_i++;
    }
    printf("inputs %ld: R mismatches %ld (FP64 %ld), q mismatches %ld (FP64 %ld), image mismatches %ld (FP64 %ld)\n",
           N, bad_r, slow_r, bad_q, slow_q, bad_i, slow_i);
    return (bad_r || bad_q || bad_i) ? 1 : 0;
}
