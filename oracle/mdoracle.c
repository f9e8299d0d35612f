/*
 * mdoracle.c -- CPU oracle for MolTwister's molecular-dynamics hot path.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
 * reference legs load this library, and only as the checker or the timed CPU baseline; the product
 * (libmtgpu.so) never calls it.
 *
 * It restates, in plain C with the same operation order, the reference's CPU code for:
 *   - the 1000-point force/potential tables (MDFF term classes, calc1DForceProfile /
 *     calc1DPotentialProfile: MolTwisterMDFFNonBonded.cpp:126-172, MolTwisterMDFFBond.cpp:133-179,
 *     MolTwisterMDFFAngle.cpp:210-257, MolTwisterMDFFDih.cpp:272-320; term formulas in _LJ.cpp:131-162,
 *     _LJ1208.cpp:131-170, _Buck.cpp:116-143, _Bond_Harm.cpp:90-110, _Morse.cpp:95-117,
 *     _Angle_Harm.cpp:94-130, _Dih_Harm.cpp:96-132, _Fourier4t.cpp:98-142);
 *   - the cell list (FunctorGenCellList.cpp:49-142) and the full neighbour list
 *     (FunctorGenNeighList.cpp:72-151);
 *   - the per-atom force/energy gather in table mode (FunctorCalcForce.cpp:95-709);
 *   - velocity-Verlet NVT/NVE with force clipping (VelVerlet.cpp:74-122), the Nose-Hoover chain
 *     (NHChain.cpp:45-113, MDLoop.cpp:29-60, Math.cpp:27-54), pbcWrap and the scalar outputs
 *     (SimulationBox.cpp:135-231), in the step order of MDLoop.cpp:128-133.
 * and adds an independent FP64 analytic force field (same gather structure, exclusions and energy
 * bookkeeping, analytic term derivatives instead of tables) as the error reference for the
 * analytic FP64 and mixed-precision GPU modes.
 *
 * Build with -ffp-contract=off so no multiply-add is fused: that is how the reference's x86-64
 * build evaluates, and it makes results identical on x86-64 and aarch64.
 * Parity pin: tests/test_oracle_golden.py checks every output here against outputs of the
 * reference itself (oracle/ref/harness.cpp) stored under tests/golden/.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_NPTS 1000
#define ORC_MAXFF 5
#define COULOMB_KF 1389.32f /* Integrators/Constants.h:40, a float literal in the reference */

/* term kinds (same codes as include/mtgpu.h) */
enum {
    K_NONE = 0,
    K_NB_LJ = 1, K_NB_LJ1208 = 2, K_NB_BUCK = 3, K_NB_LJBUCK = 4,
    K_BOND_HARM = 11, K_BOND_MORSE = 12, K_BOND_LJC = 13,
    K_ANGLE_HARM = 21, K_ANGLE_CLASS2 = 22,
    K_DIH_HARM = 31, K_DIH_FOURIER4T = 32,
    K_TABLE = 99
};

typedef struct { double x, y, z; } v3;

static v3 mk(double x, double y, double z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 scl(v3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
static double dot(v3 a, v3 b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); }
static double nrm(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static v3 crs(v3 a, v3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

/* C3DVector::moveToSameSideOfPBCAsThis (Utilities/3DVector.cpp:133-165) */
static void same_side(v3 c, v3* v, const double w[3]) {
    double dX = c.x - v->x, dY = c.y - v->y, dZ = c.z - v->z;
    dX = (dX < 0.0) ? -dX : dX;
    dY = (dY < 0.0) ? -dY : dY;
    dZ = (dZ < 0.0) ? -dZ : dZ;
    if(dX > (w[0] / 2.0)) { if(c.x > v->x) v->x += w[0]; else v->x -= w[0]; }
    if(dY > (w[1] / 2.0)) { if(c.y > v->y) v->y += w[1]; else v->y -= w[1]; }
    if(dZ > (w[2] / 2.0)) { if(c.z > v->z) v->z += w[2]; else v->z -= w[2]; }
}

/* ------------------------------------------------------------------------------------------ */
/* Geometry coefficients (FunctorCalcForce.cpp:283-424; identical in the MDFF base classes)     */
/* ------------------------------------------------------------------------------------------ */
static v3 coeff12(v3 r1, v3 r2) {
    v3 r12 = sub(r2, r1);
    double R = nrm(r12);
    double RInv = (R == 0.0) ? 1.0 / 1E-10 : 1.0 / R;
    return scl(r12, RInv);
}

static v3 coeff_ang13(v3 r1, v3 r2, v3 r3) {
    v3 r12 = sub(r1, r2);
    double R = nrm(r12);
    double RInv = (R == 0.0) ? 1.0 / 1E-10 : 1.0 / R;
    v3 K = scl(r12, RInv);
    v3 r32 = sub(r3, r2);
    double A = K.x * r32.x + K.y * r32.y + K.z * r32.z;
    double B = r32.x * r32.x + r32.y * r32.y + r32.z * r32.z;
    double sqrtB = sqrt(B);
    double sqrtB3 = (B == 0.0) ? sqrt(1E-30) : sqrtB * sqrtB * sqrtB;
    double dW_dx = (K.x * B - r32.x * A) / sqrtB3;
    double dW_dy = (K.y * B - r32.y * A) / sqrtB3;
    double dW_dz = (K.z * B - r32.z * A) / sqrtB3;
    double W = (sqrtB == 0.0) ? A / 10E-3 : A / sqrtB;
    double dDiv = sqrt(1.0 - W * W);
    double dT = (dDiv == 0.0) ? -1.0 / 1E-10 : -1.0 / dDiv;
    return mk(dT * dW_dx, dT * dW_dy, dT * dW_dz);
}

static v3 coeff_ang2(v3 r1, v3 r2, v3 r3) {
    v3 r12 = sub(r1, r2);
    v3 r32 = sub(r3, r2);
    double A = r12.x * r12.x + r12.y * r12.y + r12.z * r12.z;
    double B = r32.x * r32.x + r32.y * r32.y + r32.z * r32.z;
    double C = r12.x * r32.x + r12.y * r32.y + r12.z * r32.z;
    double AB = A * B;
    double sqrtAB = sqrt(AB);
    double sqrtAB3 = (AB == 0.0) ? sqrt(1E-30) : sqrtAB * sqrtAB * sqrtAB;
    double dW_dx = ((2.0 * r2.x - r1.x - r3.x) * AB + (r32.x * A + r12.x * B) * C) / sqrtAB3;
    double dW_dy = ((2.0 * r2.y - r1.y - r3.y) * AB + (r32.y * A + r12.y * B) * C) / sqrtAB3;
    double dW_dz = ((2.0 * r2.z - r1.z - r3.z) * AB + (r32.z * A + r12.z * B) * C) / sqrtAB3;
    double W = (sqrtAB == 0.0) ? A / 10E-3 : C / sqrtAB;
    double dDiv = sqrt(1.0 - W * W);
    double dT = (dDiv == 0.0) ? -1.0 / 1E-10 : -1.0 / dDiv;
    return mk(dT * dW_dx, dT * dW_dy, dT * dW_dz);
}

static v3 coeff_dih14(v3 r1, v3 r2, v3 r3, v3 r4) {
    v3 r21 = sub(r1, r2), r23 = sub(r3, r2);
    v3 r32 = scl(r23, -1.0);
    v3 r34 = sub(r4, r3);
    v3 n1 = crs(r23, r21);
    double n1Norm = nrm(n1);
    double n1NormInv = (n1Norm == 0.0) ? 1.0 / 1E-10 : 1.0 / n1Norm;
    v3 K = scl(n1, n1NormInv);
    double a = r32.y * r34.z - r32.z * r34.y;
    double b = r32.z * r34.x - r32.x * r34.z;
    double c = r32.x * r34.y - r32.y * r34.x;
    double A = K.x * a + K.y * b + K.z * c;
    double B = a * a + b * b + c * c;
    double sqrtBInv = (B == 0.0) ? 1.0 / 1E-20 : 1.0 / sqrt(B);
    double sqrtBInv3 = sqrtBInv * sqrtBInv * sqrtBInv;
    double W = A * sqrtBInv;
    double dW_dx = ((K.y * r32.z - K.z * r32.y) * B - (r32.z * (r32.z * r34.x - r32.x * r34.z) - r32.y * (r32.x * r34.y - r32.y * r34.x)) * A) * sqrtBInv3;
    double dW_dy = ((K.z * r32.x - K.x * r32.z) * B - (r32.x * (r32.x * r34.y - r32.y * r34.x) - r32.z * (r32.y * r34.z - r32.z * r34.y)) * A) * sqrtBInv3;
    double dW_dz = ((K.x * r32.y - K.y * r32.x) * B - (r32.y * (r32.y * r34.z - r32.z * r34.y) - r32.x * (r32.z * r34.x - r32.x * r34.z)) * A) * sqrtBInv3;
    double dv = sqrt(1.0 - W * W);
    double dT = (dv == 0.0) ? 1.0 / 1E-10 : 1.0 / dv;
    v3 o = mk(dT * dW_dx, dT * dW_dy, dT * dW_dz);
    return scl(o, -1.0);
}

static v3 coeff_dih23(v3 r1, v3 r2, v3 r3, v3 r4) {
    v3 r21 = sub(r1, r2), r23 = sub(r3, r2);
    v3 r32 = scl(r23, -1.0);
    v3 r34 = sub(r4, r3);
    double K1 = r32.z * r34.x - r32.x * r34.z;
    double K2 = r34.z - r32.z;
    double K3 = r23.z * r21.x - r23.x * r21.z;
    double K4 = r32.x * r34.y - r32.y * r34.x;
    double K5 = r32.y - r34.y;
    double K6 = r23.x * r21.y - r23.y * r21.x;
    double L1 = r32.y * r34.z - r32.z * r34.y;
    double L2 = -K2;
    double L3 = r23.y * r21.z - r23.z * r21.y;
    double L4 = K4;
    double L5 = r34.x - r32.x;
    double L6 = K6;
    double M1 = L1, M2 = -K5, M3 = L3, M4 = K1, M5 = -L5, M6 = K3;
    double A = L3 * L3 + K3 * K3 + K6 * K6;
    double B = L1 * L1 + K1 * K1 + K4 * K4;
    double C = L3 * L1 + K3 * K1 + K6 * K4;
    double AB = A * B;
    double sqrtABInv = (AB == 0.0) ? 1.0 / 1E-20 : 1.0 / sqrt(AB);
    double sqrtABInv3 = sqrtABInv * sqrtABInv * sqrtABInv;
    double W = C * sqrtABInv;
    double dC_dx = K2 * K3 + r21.y * K4 + K5 * K6 - r21.z * K1;
    double dC_dy = L2 * L3 - r21.x * L4 + L5 * L6 + r21.z * L1;
    double dC_dz = M2 * M3 + r21.x * M4 + M5 * M6 - r21.y * M1;
    double dW_dx = (dC_dx * AB - C * ((r21.y * K6 - r21.z * K3) * B + (K1 * K2 + K4 * K5) * A)) * sqrtABInv3;
    double dW_dy = (dC_dy * AB - C * ((r21.z * L3 - r21.x * L6) * B + (L1 * L2 + L4 * L5) * A)) * sqrtABInv3;
    double dW_dz = (dC_dz * AB - C * ((r21.x * M6 - r21.y * M3) * B + (M1 * M2 + M4 * M5) * A)) * sqrtABInv3;
    double dv = sqrt(1.0 - W * W);
    double dT = (dv == 0.0) ? 1.0 / 1E-10 : 1.0 / dv;
    v3 o = mk(dT * dW_dx, dT * dW_dy, dT * dW_dz);
    return scl(o, -1.0);
}

/* ------------------------------------------------------------------------------------------ */
/* Term formulas (double), returning force on r2 (pair) / r3 (angle) / r4 (dihedral) and U     */
/* ------------------------------------------------------------------------------------------ */
static double nb_pot(int kind, const double* p, v3 r1, v3 r2) {
    v3 r12 = sub(r2, r1);
    double R = nrm(r12);
    double RInv = (R == 0.0) ? 1.0 / 1E-10 : 1.0 / R;
    double RInv2 = RInv * RInv;
    if(kind == K_NB_LJ) {               /* p = eps, sigma, alpha */
        double RInv6 = RInv2 * RInv2 * RInv2, RInv12 = RInv6 * RInv6;
        double s2 = p[1] * p[1], s6 = s2 * s2 * s2, s12 = s6 * s6;
        return 4.0 * p[0] * (s12 * RInv12 - p[2] * s6 * RInv6);
    }
    if(kind == K_NB_LJ1208) {
        double RInv4 = RInv2 * RInv2, RInv6 = RInv4 * RInv2, RInv8 = RInv4 * RInv4, RInv12 = RInv6 * RInv6;
        double s2 = p[1] * p[1], s4 = s2 * s2, s6 = s4 * s2, s8 = s4 * s4, s12 = s6 * s6;
        (void)RInv6;
        return 4.0 * p[0] * (s12 * RInv12 - p[2] * s8 * RInv8);
    }
    if(kind == K_NB_BUCK) {             /* p = A, rho, C */
        double RInv4 = RInv2 * RInv2, RInv6 = RInv4 * RInv2;
        double rhoInv = (p[1] == 0.0) ? 1E-10 : 1.0 / p[1];
        return p[0] * exp(-R * rhoInv) - p[2] * RInv6;
    }
    return 0.0;
}

static double nb_force_x(int kind, const double* p, v3 r1, v3 r2) {
    v3 r12 = sub(r2, r1);
    double R = nrm(r12);
    double RInv = (R == 0.0) ? 1.0 / 1E-10 : 1.0 / R;
    double RInv2 = RInv * RInv;
    double g = 0.0;
    if(kind == K_NB_LJ) {
        double RInv6 = RInv2 * RInv2 * RInv2, RInv12 = RInv6 * RInv6;
        double s2 = p[1] * p[1], s6 = s2 * s2 * s2, s12 = s6 * s6;
        g = 4.0 * p[0] * RInv2 * (12.0 * s12 * RInv12 - 6.0 * p[2] * s6 * RInv6);
    } else if(kind == K_NB_LJ1208) {
        double RInv4 = RInv2 * RInv2, RInv6 = RInv4 * RInv2, RInv8 = RInv4 * RInv4, RInv12 = RInv6 * RInv6;
        double s2 = p[1] * p[1], s4 = s2 * s2, s6 = s4 * s2, s8 = s4 * s4, s12 = s6 * s6;
        g = 4.0 * p[0] * RInv2 * (12.0 * s12 * RInv12 - 8.0 * p[2] * s8 * RInv8);
    } else if(kind == K_NB_BUCK) {
        double RInv4 = RInv2 * RInv2, RInv6 = RInv4 * RInv2;
        double rhoInv = (p[1] == 0.0) ? 1E-10 : 1.0 / p[1];
        g = RInv2 * (p[0] * R * rhoInv * exp(-R * rhoInv) - 6.0 * p[2] * RInv6);
    } else {
        return 0.0;
    }
    return r12.x * g;
}

static double bond_pot(int kind, const double* p, v3 r1, v3 r2) {
    v3 r12 = sub(r2, r1);
    double R = nrm(r12);
    if(kind == K_BOND_HARM) { double d = R - p[1]; return p[0] * d * d; }            /* k, r0 */
    if(kind == K_BOND_MORSE) { double d = R - p[2]; double P = (1.0 - exp(-p[1] * d)); return p[0] * P * P; } /* D, alpha, r0 */
    return 0.0;
}

static double bond_force_x(int kind, const double* p, v3 r1, v3 r2) {
    v3 r12 = sub(r2, r1);
    double R = nrm(r12);
    double RInv = (R == 0.0) ? 1.0 / 1E-10 : 1.0 / R;
    double g;
    if(kind == K_BOND_HARM) { double d = R - p[1]; g = -2.0 * p[0] * d * RInv; }
    else if(kind == K_BOND_MORSE) { double d = R - p[2]; double E = exp(-p[1] * d); g = -2.0 * p[0] * p[1] * RInv * E * (1.0 - E); }
    else return 0.0;
    return r12.x * g;
}

/* angle Harm: p = k, theta0 [deg], toRad */
static double angle_theta(v3 r1, v3 r2, v3 r3) {
    v3 r21 = sub(r1, r2), r23 = sub(r3, r2);
    double R21 = nrm(r21), R23 = nrm(r23);
    double R21Inv = (R21 == 0.0) ? 1.0 / 1E-10 : 1.0 / R21;
    double R23Inv = (R23 == 0.0) ? 1.0 / 1E-10 : 1.0 / R23;
    double cosT = dot(r21, r23) * (R21Inv * R23Inv);
    return acos(cosT);
}

static double angle_pot(int kind, const double* p, v3 r1, v3 r2, v3 r3) {
    if(kind != K_ANGLE_HARM) return 0.0;
    double d = angle_theta(r1, r2, r3) - p[1] * p[2];
    return p[0] * d * d;
}

static double angle_force3_x(int kind, const double* p, v3 r1, v3 r2, v3 r3) {
    if(kind != K_ANGLE_HARM) return 0.0;
    double d = angle_theta(r1, r2, r3) - p[1] * p[2];
    v3 c3 = coeff_ang13(r1, r2, r3);
    double dU = -2.0 * p[0] * d;
    return c3.x * dU;
}

static double dih_phi(v3 r1, v3 r2, v3 r3, v3 r4) {
    v3 r21 = sub(r1, r2), r23 = sub(r3, r2);
    v3 r32 = scl(r23, -1.0);
    v3 r34 = sub(r4, r3);
    v3 n1 = crs(r23, r21), n2 = crs(r32, r34);
    double n1n2 = nrm(n1) * nrm(n2);
    double c = (n1n2 == 0.0) ? dot(n1, n2) / 1E-20 : dot(n1, n2) / n1n2;
    return acos(c);
}

static double dih_pot(int kind, const double* p, v3 r1, v3 r2, v3 r3, v3 r4) {
    double phi = dih_phi(r1, r2, r3, r4);
    if(kind == K_DIH_HARM) return p[0] * (1.0 + (double)(int)p[1] * cos((double)(int)p[2] * phi));
    if(kind == K_DIH_FOURIER4T) {
        double U1 = p[0] * (1.0 + cos(phi)), U2 = p[1] * (1.0 - cos(2.0 * phi));
        double U3 = p[2] * (1.0 + cos(3.0 * phi)), U4 = p[3] * (1.0 - cos(4.0 * phi));
        return 0.5 * (U1 + U2 + U3 + U4);
    }
    return 0.0;
}

static double dih_dU(int kind, const double* p, double phi) {
    if(kind == K_DIH_HARM) { int D = (int)p[1], N = (int)p[2]; return -p[0] * (double)(D * N) * sin((double)N * phi); }
    if(kind == K_DIH_FOURIER4T) {
        double a = -0.5 * p[0] * sin(phi), b = p[1] * sin(2.0 * phi);
        double c = -1.5 * p[2] * sin(3.0 * phi), d = 2.0 * p[3] * sin(4.0 * phi);
        return a + b + c + d;
    }
    return 0.0;
}

static double dih_force4_x(int kind, const double* p, v3 r1, v3 r2, v3 r3, v3 r4) {
    double phi = dih_phi(r1, r2, r3, r4);
    double dU = dih_dU(kind, p, phi);
    v3 c4 = coeff_dih14(r1, r2, r3, r4);
    return c4.x * dU;
}

/* ------------------------------------------------------------------------------------------ */
/* Tables: out[3*i] = x, out[3*i+1] = -dU/dx (as F_x / (dx/dx_x)), out[3*i+2] = U               */
/* ------------------------------------------------------------------------------------------ */
int orc_profile_nb(int kind, const double* p, float r0, float r1, int npts, float* out) {
    float d = (r1 - r0) / (float)(npts - 1);
    for(int i = 0; i < npts; i++) {
        float r = r0 + (float)i * d;
        v3 a = mk(0, 0, 0), b = mk((double)r, 0, 0);
        double fx = nb_force_x(kind, p, a, b);
        v3 c = coeff12(a, b);
        out[3 * i] = r;
        out[3 * i + 1] = (float)((c.x != 0.0) ? fx / c.x : 0.0);
        out[3 * i + 2] = (float)nb_pot(kind, p, a, b);
    }
    return 0;
}

int orc_profile_bond(int kind, const double* p, float r0, float r1, int npts, float* out) {
    float d = (r1 - r0) / (float)(npts - 1);
    for(int i = 0; i < npts; i++) {
        float r = r0 + (float)i * d;
        v3 a = mk(0, 0, 0), b = mk((double)r, 0, 0);
        double fx = bond_force_x(kind, p, a, b);
        v3 c = coeff12(a, b);
        out[3 * i] = r;
        out[3 * i + 1] = (float)((c.x != 0.0) ? fx / c.x : 0.0);
        out[3 * i + 2] = (float)bond_pot(kind, p, a, b);
    }
    return 0;
}

int orc_profile_angle(int kind, const double* p, float t0, float t1, int npts, float* out) {
    float d = (t1 - t0) / (float)(npts - 1);
    for(int i = 0; i < npts; i++) {
        float t = t0 + (float)i * d;
        v3 a = mk(-1.0, 0, 0), b = mk(0, 0, 0), c3 = mk(-cos((double)t), sin((double)t), 0.0);
        double fx = angle_force3_x(kind, p, a, b, c3);
        v3 c = coeff_ang13(a, b, c3);
        out[3 * i] = t;
        out[3 * i + 1] = (float)((c.x != 0.0) ? fx / c.x : 0.0);
        out[3 * i + 2] = (float)angle_pot(kind, p, a, b, c3);
    }
    return 0;
}

int orc_profile_dih(int kind, const double* p, float t0, float t1, int npts, float* out) {
    float d = (t1 - t0) / (float)(npts - 1);
    for(int i = 0; i < npts; i++) {
        float t = t0 + (float)i * d;
        v3 a = mk(0, 1.0, 0), b = mk(0, 0, 0), c3 = mk(0, 0, 1.0), d4 = mk(sin((double)t), cos((double)t), 1.0);
        double fx = dih_force4_x(kind, p, a, b, c3, d4);
        v3 c = coeff_dih14(a, b, c3, d4);
        out[3 * i] = t;
        out[3 * i + 1] = (float)((c.x != 0.0) ? fx / c.x : 0.0);
        out[3 * i + 2] = (float)dih_pot(kind, p, a, b, c3, d4);
    }
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Cell list: CFunctorGenCellList::operator() + kernelAssembleList (FunctorGenCellList.cpp)     */
/* box is float (CCellList::updatePBC: low = -L/2 in float, MDFFMatrices.cpp:67-76)             */
/* ------------------------------------------------------------------------------------------ */
int orc_cell_list(int n, const double* r, const float* L, int nx, int ny, int nz,
                  int* atom_cell /* n*3 */, int* cell_ptr /* ncell*2: first, count */, int* cell_list /* n */) {
    const float wx = L[0], wy = L[1], wz = L[2];
    const float lx = -wx / 2.0f, ly = -wy / 2.0f, lz = -wz / 2.0f;
    const int ncell = nx * ny * nz;
    for(int i = 0; i < n; i++) {
        int ix = (int)floor((r[3 * i] - (double)lx) * (double)nx / (double)wx);
        int iy = (int)floor((r[3 * i + 1] - (double)ly) * (double)ny / (double)wy);
        int iz = (int)floor((r[3 * i + 2] - (double)lz) * (double)nz / (double)wz);
        ix = (ix < 0) ? 0 : ((ix >= nx) ? nx - 1 : ix);
        iy = (iy < 0) ? 0 : ((iy >= ny) ? ny - 1 : iy);
        iz = (iz < 0) ? 0 : ((iz >= nz) ? nz - 1 : iz);
        atom_cell[3 * i] = ix; atom_cell[3 * i + 1] = iy; atom_cell[3 * i + 2] = iz;
    }
    for(int c = 0; c < ncell; c++) { cell_ptr[2 * c] = -1; cell_ptr[2 * c + 1] = 0; }
    for(int i = 0; i < n; i++) {
        int c = atom_cell[3 * i] + nx * (atom_cell[3 * i + 1] + atom_cell[3 * i + 2] * ny);
        cell_ptr[2 * c + 1]++;
    }
    int next = 0;
    for(int c = 0; c < ncell; c++) {
        if(cell_ptr[2 * c + 1] != 0) { cell_ptr[2 * c] = next; next += cell_ptr[2 * c + 1]; cell_ptr[2 * c + 1] = 0; }
    }
    for(int i = 0; i < n; i++) {
        int c = atom_cell[3 * i] + nx * (atom_cell[3 * i + 1] + atom_cell[3 * i + 2] * ny);
        int e = cell_ptr[2 * c] + cell_ptr[2 * c + 1];
        cell_list[e] = i;
        cell_ptr[2 * c + 1]++;
    }
    return 0;
}

/* Full neighbour list, reference order (FunctorGenNeighList.cpp:72-151).  Counts are always
 * complete; list entries beyond maxn are not written.  Returns the largest count. */
int orc_neigh_list(int n, const double* r, const float* L, float rc, int nx, int ny, int nz,
                   const int* atom_cell, const int* cell_ptr, const int* cell_list,
                   int maxn, int* count, int* list) {
    float rc2f = rc; rc2f *= rc2f;
    const double rc2 = (double)rc2f;
    const float lx = -L[0] / 2.0f, ly = -L[1] / 2.0f, lz = -L[2] / 2.0f;
    /* pbc_ of the functor: rLow = double(low), rHigh = double(low + width) computed in float */
    const double w[3] = {(double)(lx + L[0]) - (double)lx, (double)(ly + L[1]) - (double)ly, (double)(lz + L[2]) - (double)lz};
    int maxc = 0;
    /* atoms are independent: each writes only its own count and row */
#pragma omp parallel for schedule(static, 64) reduction(max : maxc)
    for(int k = 0; k < n; k++) {
        int c = 0;
        double x0 = r[3 * k], y0 = r[3 * k + 1], z0 = r[3 * k + 2];
        for(int ix = atom_cell[3 * k] - 1; ix <= atom_cell[3 * k] + 1; ix++) {
            int Ix = (ix >= 0) ? ((ix < nx) ? ix : 0) : nx - 1;
            for(int iy = atom_cell[3 * k + 1] - 1; iy <= atom_cell[3 * k + 1] + 1; iy++) {
                int Iy = (iy >= 0) ? ((iy < ny) ? iy : 0) : ny - 1;
                for(int iz = atom_cell[3 * k + 2] - 1; iz <= atom_cell[3 * k + 2] + 1; iz++) {
                    int Iz = (iz >= 0) ? ((iz < nz) ? iz : 0) : nz - 1;
                    int cell = Ix + nx * (Iy + Iz * ny);
                    int cnt = cell_ptr[2 * cell + 1], first = cell_ptr[2 * cell];
                    for(int e = 0; e < cnt; e++) {
                        int j = cell_list[first + e];
                        double dX = x0 - r[3 * j], dY = y0 - r[3 * j + 1], dZ = z0 - r[3 * j + 2];
                        dX = (dX < 0.0) ? -dX : dX;
                        dY = (dY < 0.0) ? -dY : dY;
                        dZ = (dZ < 0.0) ? -dZ : dZ;
                        if(dX > (w[0] / 2.0)) dX = w[0] - dX;
                        if(dY > (w[1] / 2.0)) dY = w[1] - dY;
                        if(dZ > (w[2] / 2.0)) dZ = w[2] - dZ;
                        double d2 = dX * dX + dY * dY + dZ * dZ;
                        if(d2 < rc2) {
                            if(j == k) continue;
                            if(c < maxn) list[(size_t)k * maxn + c] = j;
                            c++;
                        }
                    }
                }
            }
        }
        count[k] = c;
        if(c > maxc) maxc = c;
    }
    return maxc;
}

/* ------------------------------------------------------------------------------------------ */
/* System description                                                                          */
/* ------------------------------------------------------------------------------------------ */
typedef struct orc_sys {
    int n, ntypes;
    const double* r;          /* n*3 positions */
    const float* q;           /* n charges (float, as CMDFFMatrices::CAtom::q_) */
    const double* m;          /* n masses */
    const int* type;          /* n */
    const int* mol;           /* n */
    const int* mobile;        /* n */
    double box[3];            /* LmaxX_, LmaxY_, LmaxZ_ (double) */
    float rc, shell, fcut;
    float scale12, scale13, scale14, scale1N;
    const float* nb_tab;      /* [((row*T + col)*5 + ff)*1000 + pt]*3 */
    const int* nb_cnt;        /* [row*T + col] */
    const float* bond_tab;    /* [type*1000 + pt]*3 */
    const float* angle_tab;
    const float* dih_tab;
    const int* bptr; const int* bj; const int* bt;                          /* per-atom bonds */
    const int* aptr; const int* ai; const int* aj; const int* at; const int* acen;
    const int* dptr; const int* di; const int* dj; const int* dl; const int* dt; const int* dcen;
    const int* nb_kind; const double* nb_par;   /* [(row*T+col)*5+ff], params[4] */
    const int* bond_kind; const double* bond_par;
    const int* angle_kind; const double* angle_par;
    const int* dih_kind; const double* dih_par;
    int coulomb_mode;         /* 0 all pairs minimum image (reference), 1 truncated, 2 shifted force at coulomb_rc */
    double coulomb_rc;
    const double* qd;         /* n charges in FP64 (analytic mode) */
    int lj_shift;             /* analytic mode: 1 shift LJ energies to zero at the cutoff, 2 shift forces too */
} orc_sys;

/* FunctorCalcForce::scaleForcesAndPotentials (FunctorCalcForce.cpp:95-157) as a factor */
static float exclusion_scale(const orc_sys* s, int k, int i, int* applies) {
    *applies = 1;
    for(int e = s->bptr[k]; e < s->bptr[k + 1]; e++) if(s->bj[e] == i) return s->scale12;
    for(int e = s->aptr[k]; e < s->aptr[k + 1]; e++) if(!s->acen[e] && s->aj[e] == i) return s->scale13;
    for(int e = s->dptr[k]; e < s->dptr[k + 1]; e++) if(!s->dcen[e] && s->dl[e] == i) return s->scale14;
    int mi = s->mol[i], mk_ = s->mol[k];
    if(mi >= 0 && mk_ >= 0 && mi == mk_) return s->scale1N;
    *applies = 0;
    return 1.0f;
}

/* x86-64 semantics of (int) on a float: NaN and out-of-range give INT_MIN */
static int f2i(float x) {
    if(!(x > -2147483648.0f && x < 2147483648.0f)) return INT32_MIN;
    return (int)x;
}

static int table_index(float x, const float* tab) {
    float delta = (tab[3 * (ORC_NPTS - 1)] - tab[0]) / (float)(ORC_NPTS - 1);
    return f2i((x - tab[0]) / delta);
}

static float interp(float r, float x1, float y1, float x2, float y2) {
    float denom = x1 - x2;
    if(denom == 0.0f) denom = 3.0f * FLT_MIN;
    float a = (y1 - y2) / denom;
    float b = y1 - a * x1;
    return (a * r + b);
}

static float calc_angle_f(v3 rk, v3 ri, v3 rj) {
    v3 rik = sub(rk, ri), rij = sub(rj, ri);
    float dp = (float)dot(rik, rij);
    float RR = (float)nrm(rik) * (float)nrm(rij);
    float c = (RR != 0.0f) ? dp / RR : 1.0f;
    return (float)acos((double)c);
}

static float calc_dih_f(v3 rk, v3 ri, v3 rj, v3 rl) {
    v3 rik = sub(rk, ri), rij = sub(rj, ri), rjl = sub(rl, rj);
    v3 n1 = crs(rik, rij), n2 = crs(rij, rjl);
    float dp = (float)dot(n1, n2);
    float nn = (float)nrm(n1) * (float)nrm(n2);
    float c = (nn != 0.0f) ? dp / nn : 1.0f;
    if(c < -1.0f) c = -1.0f;
    if(c > 1.0f) c = 1.0f;
    return (float)acos((double)c);
}

/* ------------------------------------------------------------------------------------------ */
/* Table-mode forces: CFunctorCalcForce::operator() (FunctorCalcForce.cpp:159-281)             */
/* F = Fpi here (no Ewald).  Lx, Ly, Lz are the float box of the functor constructor.         */
/* ------------------------------------------------------------------------------------------ */
int orc_forces_ref(const orc_sys* s, const int* ncount, const int* nlist, int maxn, double* F, float* U) {
    const float Lf[3] = {(float)s->box[0], (float)s->box[1], (float)s->box[2]};
    const double w[3] = {(double)Lf[0] / 2.0 - (-(double)Lf[0] / 2.0), (double)Lf[1] / 2.0 - (-(double)Lf[1] / 2.0),
                         (double)Lf[2] / 2.0 - (-(double)Lf[2] / 2.0)};
    const int T = s->ntypes;
    /* each atom sums its own terms in the reference's order, so the threads change no result */
#pragma omp parallel for schedule(dynamic, 16)
    for(int k = 0; k < s->n; k++) {
        v3 Fk = mk(0, 0, 0);
        float Uk = 0.0f;
        F[3 * k] = F[3 * k + 1] = F[3 * k + 2] = 0.0;
        U[k] = 0.0f;
        if(!s->mobile[k]) continue;
        v3 rk = mk(s->r[3 * k], s->r[3 * k + 1], s->r[3 * k + 2]);
        /* bonds */
        for(int e = s->bptr[k]; e < s->bptr[k + 1]; e++) {
            int i = s->bj[e];
            v3 ri = mk(s->r[3 * i], s->r[3 * i + 1], s->r[3 * i + 2]);
            same_side(rk, &ri, w);
            const float* tab = s->bond_tab + (size_t)s->bt[e] * ORC_NPTS * 3;
            float rr = (float)nrm(sub(rk, ri));
            int idx = table_index(rr, tab);
            float md = 0.0f;
            if(idx >= 0 && idx < ORC_NPTS - 1) {
                const float* p1 = tab + 3 * idx; const float* p2 = p1 + 3;
                md += interp(rr, p1[0], p1[1], p2[0], p2[1]);
                if(i > k) Uk += interp(rr, p1[0], p1[2], p2[0], p2[2]);
            }
            v3 c = coeff12(ri, rk);
            v3 f = scl(c, (double)md);
            Fk.x += f.x; Fk.y += f.y; Fk.z += f.z;
        }
        /* angles */
        for(int e = s->aptr[k]; e < s->aptr[k + 1]; e++) {
            v3 ri = mk(s->r[3 * s->ai[e]], s->r[3 * s->ai[e] + 1], s->r[3 * s->ai[e] + 2]);
            v3 rj = mk(s->r[3 * s->aj[e]], s->r[3 * s->aj[e] + 1], s->r[3 * s->aj[e] + 2]);
            same_side(rk, &ri, w);
            same_side(rk, &rj, w);
            const float* tab = s->angle_tab + (size_t)s->at[e] * ORC_NPTS * 3;
            v3 f;
            if(s->acen[e]) {
                /* calcForceAngularOn_r_i(r_k := ri, r_i := rk, r_j := rj) */
                float th = calc_angle_f(ri, rk, rj);
                int idx = table_index(th, tab);
                float md = 0.0f;
                if(idx >= 0 && idx < ORC_NPTS - 1) {
                    const float* p1 = tab + 3 * idx; const float* p2 = p1 + 3;
                    md += interp(th, p1[0], p1[1], p2[0], p2[1]);
                    Uk += interp(th, p1[0], p1[2], p2[0], p2[2]);
                }
                f = scl(coeff_ang2(rj, rk, ri), (double)md);
            } else {
                float th = calc_angle_f(rk, ri, rj);
                int idx = table_index(th, tab);
                float md = 0.0f;
                if(idx >= 0 && idx < ORC_NPTS - 1) {
                    const float* p1 = tab + 3 * idx; const float* p2 = p1 + 3;
                    md += interp(th, p1[0], p1[1], p2[0], p2[1]);
                }
                f = scl(coeff_ang13(rj, ri, rk), (double)md);
            }
            Fk.x += f.x; Fk.y += f.y; Fk.z += f.z;
        }
        /* dihedrals */
        for(int e = s->dptr[k]; e < s->dptr[k + 1]; e++) {
            v3 ri = mk(s->r[3 * s->di[e]], s->r[3 * s->di[e] + 1], s->r[3 * s->di[e] + 2]);
            v3 rj = mk(s->r[3 * s->dj[e]], s->r[3 * s->dj[e] + 1], s->r[3 * s->dj[e] + 2]);
            v3 rl = mk(s->r[3 * s->dl[e]], s->r[3 * s->dl[e] + 1], s->r[3 * s->dl[e] + 2]);
            same_side(rk, &ri, w);
            same_side(rk, &rj, w);
            same_side(rk, &rl, w);
            const float* tab = s->dih_tab + (size_t)s->dt[e] * ORC_NPTS * 3;
            v3 f;
            if(s->dcen[e]) {
                float th = calc_dih_f(ri, rk, rj, rl);
                int idx = table_index(th, tab);
                float md = 0.0f;
                if(idx >= 0 && idx < ORC_NPTS - 1) {
                    const float* p1 = tab + 3 * idx; const float* p2 = p1 + 3;
                    md += interp(th, p1[0], p1[1], p2[0], p2[1]);
                    Uk += 0.5f * interp(th, p1[0], p1[2], p2[0], p2[2]);
                }
                f = scl(coeff_dih23(rl, rj, rk, ri), (double)md);
            } else {
                float th = calc_dih_f(rk, ri, rj, rl);
                int idx = table_index(th, tab);
                float md = 0.0f;
                if(idx >= 0 && idx < ORC_NPTS - 1) {
                    const float* p1 = tab + 3 * idx; const float* p2 = p1 + 3;
                    md += interp(th, p1[0], p1[1], p2[0], p2[1]);
                }
                f = scl(coeff_dih14(rl, rj, ri, rk), (double)md);
            }
            Fk.x += f.x; Fk.y += f.y; Fk.z += f.z;
        }
        /* short range, neighbour-list order */
        for(int e = 0; e < ncount[k]; e++) {
            int i = nlist[(size_t)k * maxn + e];
            float u = 0.0f;
            v3 ri = mk(s->r[3 * i], s->r[3 * i + 1], s->r[3 * i + 2]);
            same_side(rk, &ri, w);
            v3 f = mk(0, 0, 0);
            float rr = (float)nrm(sub(rk, ri));
            if(!(rr < 1E-3f)) {
                float sum = 0.0f;
                int pair = s->type[k] * T + s->type[i];
                int cnt = s->nb_cnt[pair];
                for(int ff = 0; ff < cnt; ff++) {
                    const float* tab = s->nb_tab + ((size_t)pair * ORC_MAXFF + ff) * ORC_NPTS * 3;
                    int idx = table_index(rr, tab);
                    if(idx >= 0 && idx < ORC_NPTS - 1) {
                        const float* p1 = tab + 3 * idx; const float* p2 = p1 + 3;
                        sum += interp(rr, p1[0], p1[1], p2[0], p2[1]);
                        if(i > k) u += interp(rr, p1[0], p1[2], p2[0], p2[2]);
                    }
                }
                f = scl(coeff12(ri, rk), (double)sum);
            }
            int ap;
            float sc = exclusion_scale(s, k, i, &ap);
            if(ap) { f = scl(f, (double)sc); u *= sc; }
            Fk.x += f.x; Fk.y += f.y; Fk.z += f.z;
            Uk += u;
        }
        const float qk = s->q[k];
        if(s->coulomb_mode != 0) {
            /* Not in the reference: Coulomb cut off at coulomb_rc (<= the list cutoff), taken over
             * the same neighbour list with the reference's pair arithmetic (float R, double K),
             * plain (mode 1) or shifted-force (mode 2).  It lets the CPU baseline run the same
             * physics as the production GPU modes. */
            const double rq = s->coulomb_rc;
            for(int e = 0; e < ncount[k]; e++) {
                int i = nlist[(size_t)k * maxn + e];
                float u = 0.0f;
                v3 ri = mk(s->r[3 * i], s->r[3 * i + 1], s->r[3 * i + 2]);
                same_side(rk, &ri, w);
                v3 rv = sub(rk, ri);
                float R = (float)nrm(rv);
                if(!((double)R < rq) || R == 0.0f) continue;
                double K = (double)(COULOMB_KF * qk * s->q[i]);
                double Rd = (double)R, g;
                if(s->coulomb_mode == 2) {
                    g = K * (1.0 / (Rd * Rd) - 1.0 / (rq * rq)) / Rd;
                    if(i > k) u += (float)(K * (1.0 / Rd - 1.0 / rq + (Rd - rq) / (rq * rq)));
                } else {
                    g = K / (Rd * Rd * Rd);
                    if(i > k) u += (float)K / R;
                }
                v3 f = scl(rv, g);
                int ap;
                float sc = exclusion_scale(s, k, i, &ap);
                if(ap) { f = scl(f, (double)sc); u *= sc; }
                Fk.x += f.x; Fk.y += f.y; Fk.z += f.z;
                Uk += u;
            }
            F[3 * k] = Fk.x; F[3 * k + 1] = Fk.y; F[3 * k + 2] = Fk.z;
            U[k] = Uk;
            continue;
        }
        /* Coulomb, all atoms (FunctorCalcForce.cpp:258-278, 514-535) */
        for(int i = 0; i < s->n; i++) {
            float u = 0.0f;
            v3 ri = mk(s->r[3 * i], s->r[3 * i + 1], s->r[3 * i + 2]);
            same_side(rk, &ri, w);
            v3 rv = sub(rk, ri);
            float qi = s->q[i];
            float R = (float)nrm(rv);
            double R3 = (double)(R * R * R);
            double K = (double)(COULOMB_KF * qk * qi);
            if((i > k) && (R != 0.0f)) u += (float)K / R;
            v3 f = (R3 != 0.0) ? scl(rv, K / R3) : mk(0, 0, 0);
            int ap;
            float sc = exclusion_scale(s, k, i, &ap);
            if(ap) { f = scl(f, (double)sc); u *= sc; }
            Fk.x += f.x; Fk.y += f.y; Fk.z += f.z;
            Uk += u;
        }
        F[3 * k] = Fk.x; F[3 * k + 1] = Fk.y; F[3 * k + 2] = Fk.z;
        U[k] = Uk;
    }
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Analytic FP64 forces.  Same gather structure, exclusions and per-atom energy bookkeeping as */
/* the table mode, with exact term derivatives.  Minimum image by per-axis rounding.           */
/* Dihedrals: the MD path measures the supplement of the standard (cis = 0) dihedral          */
/* (FunctorCalcForce.cpp:442-455) and its tables are built on a geometry whose abscissa is the */
/* supplement as well (MolTwisterMDFFDih.cpp:279-291); the two flips cancel, so the reference */
/* applies the term formula U(phi) to the standard unsigned dihedral phi.                      */
/* U[k] is the per-atom energy (double); virial W = sum over k of F_k . r_k is not used.       */
/* ------------------------------------------------------------------------------------------ */
static v3 minimg(v3 d, const double* L) {
    d.x -= L[0] * rint(d.x / L[0]);
    d.y -= L[1] * rint(d.y / L[1]);
    d.z -= L[2] * rint(d.z / L[2]);
    return d;
}

/* -dU/dr for one analytic pair term and U */
/* LJ/LJ1208 p = {eps, sigma, alpha, rc}: rc > 0 is the term's own cutoff (new option of the
 * production modes); shift 1 shifts the energy to zero at the cutoff in force (rc, else rglob),
 * shift 2 shifts the force as well. */
static void nb_analytic(int kind, const double* p, double R, double rglob, int shift, double* mdUdr, double* u) {
    if(kind == K_NB_LJ || kind == K_NB_LJ1208) {
        const double rct = p[3] > 0.0 ? p[3] : rglob;
        *u = 0.0; *mdUdr = 0.0;
        if(p[3] > 0.0 && R >= p[3]) return;
        double srn, sr12;
        const double n = (kind == K_NB_LJ) ? 6.0 : 8.0;
        double sr2 = (p[1] * p[1]) / (R * R);
        if(kind == K_NB_LJ) { srn = sr2 * sr2 * sr2; sr12 = srn * srn; }
        else { double sr4 = sr2 * sr2; srn = sr4 * sr4; sr12 = srn * sr4; }
        *u = 4.0 * p[0] * (sr12 - p[2] * srn);
        *mdUdr = 4.0 * p[0] * (12.0 * sr12 - n * p[2] * srn) / R;
        if(shift) {
            double c2 = (p[1] * p[1]) / (rct * rct), cn, c12;
            if(kind == K_NB_LJ) { cn = c2 * c2 * c2; c12 = cn * cn; }
            else { double c4 = c2 * c2; cn = c4 * c4; c12 = cn * c4; }
            *u -= 4.0 * p[0] * (c12 - p[2] * cn);
            if(shift == 2) {   /* force shifted: F - F(rc), U - U(rc) + (r - rc) F(rc) */
                const double Fc = 4.0 * p[0] * (12.0 * c12 - n * p[2] * cn) / rct;
                *mdUdr -= Fc;
                *u += (R - rct) * Fc;
            }
        }
    } else if(kind == K_NB_BUCK) {
        double e = p[0] * exp(-R / p[1]), r6 = 1.0 / (R * R * R * R * R * R);
        *u = e - p[2] * r6;
        *mdUdr = e / p[1] - 6.0 * p[2] * r6 / R;
    } else { *u = 0.0; *mdUdr = 0.0; }
}

/* FP64 analytic forces and per-atom energies; with W also each atom's share of the virial
 * sum_a r_a . F_a: (r_i - r_j) . F_i once per pair (on the lower index), and for every bonded term
 * (r_k - r_X) . F_k with X the term's lowest-index atom (bonds, dihedrals) or its centre (angles),
 * which sums over the term's atoms to the term's virial because its forces sum to zero. */
static int forces_fp64(const orc_sys* s, double rcut, double* F, double* U, double* W);

int orc_forces_fp64(const orc_sys* s, double rcut, double* F, double* U) { return forces_fp64(s, rcut, F, U, NULL); }

int orc_forces_fp64_vir(const orc_sys* s, double rcut, double* F, double* U, double* W) {
    return forces_fp64(s, rcut, F, U, W);
}

static int forces_fp64(const orc_sys* s, double rcut, double* F, double* U, double* W) {
    const double* L = s->box;
    const int T = s->ntypes;
    const double rc2 = rcut * rcut;
    const double crc2 = s->coulomb_rc * s->coulomb_rc;
#pragma omp parallel for schedule(dynamic, 16)
    for(int k = 0; k < s->n; k++) {
        double fx = 0, fy = 0, fz = 0, uk = 0, wk = 0;
        F[3 * k] = F[3 * k + 1] = F[3 * k + 2] = 0.0;
        U[k] = 0.0;
        if(W) W[k] = 0.0;
        if(!s->mobile[k]) continue;
        v3 rk = mk(s->r[3 * k], s->r[3 * k + 1], s->r[3 * k + 2]);
        for(int e = s->bptr[k]; e < s->bptr[k + 1]; e++) {
            int i = s->bj[e];
            v3 d = minimg(sub(rk, mk(s->r[3 * i], s->r[3 * i + 1], s->r[3 * i + 2])), L);
            double R = nrm(d);
            const double* p = s->bond_par + 4 * s->bt[e];
            int kind = s->bond_kind[s->bt[e]];
            double md = 0, u = 0;
            if(kind == K_BOND_HARM) { md = -2.0 * p[0] * (R - p[1]); u = p[0] * (R - p[1]) * (R - p[1]); }
            else if(kind == K_BOND_MORSE) { double E = exp(-p[1] * (R - p[2])); md = -2.0 * p[0] * p[1] * E * (1.0 - E); u = p[0] * (1.0 - E) * (1.0 - E); }
            fx += md * d.x / R; fy += md * d.y / R; fz += md * d.z / R;
            if(i > k) uk += u;
            if(k > i) wk += md * R;
        }
        for(int e = s->aptr[k]; e < s->aptr[k + 1]; e++) {
            /* theta at the centre; gradient of theta wrt each atom */
            int c, a1, a3;
            if(s->acen[e]) { c = k; a1 = s->ai[e]; a3 = s->aj[e]; }
            else { c = s->ai[e]; a1 = k; a3 = s->aj[e]; }
            v3 rc_ = mk(s->r[3 * c], s->r[3 * c + 1], s->r[3 * c + 2]);
            v3 u1 = minimg(sub(mk(s->r[3 * a1], s->r[3 * a1 + 1], s->r[3 * a1 + 2]), rc_), L);
            v3 u3 = minimg(sub(mk(s->r[3 * a3], s->r[3 * a3 + 1], s->r[3 * a3 + 2]), rc_), L);
            double n1 = nrm(u1), n3 = nrm(u3);
            double cs = dot(u1, u3) / (n1 * n3);
            if(cs > 1.0) cs = 1.0;
            if(cs < -1.0) cs = -1.0;
            double th = acos(cs), sn = sqrt(1.0 - cs * cs);
            const double* p = s->angle_par + 4 * s->at[e];
            double dU = 0, u = 0;
            if(s->angle_kind[s->at[e]] == K_ANGLE_HARM) { double dd = th - p[1] * p[2]; dU = 2.0 * p[0] * dd; u = p[0] * dd * dd; }
            if(sn < 1e-12) sn = 1e-12;
            /* dtheta/du1 = -(u3/(n1 n3) - cs u1/n1^2) / sin */
            v3 g1 = scl(sub(scl(u3, 1.0 / (n1 * n3)), scl(u1, cs / (n1 * n1))), -1.0 / sn);
            v3 g3 = scl(sub(scl(u1, 1.0 / (n1 * n3)), scl(u3, cs / (n3 * n3))), -1.0 / sn);
            v3 g;
            if(s->acen[e]) { g = mk(-g1.x - g3.x, -g1.y - g3.y, -g1.z - g3.z); uk += u; }
            else {
                g = g1;
                wk -= dU * dot(u1, g1);      /* (r_k - r_centre) . F_k */
            }
            fx -= dU * g.x; fy -= dU * g.y; fz -= dU * g.z;
        }
        for(int e = s->dptr[k]; e < s->dptr[k + 1]; e++) {
            /* atoms in dihedral order a-b-c-d; k is a (end) or b (centre) in the per-atom list */
            int a, b, c, d;
            if(s->dcen[e]) { a = s->di[e]; b = k; c = s->dj[e]; d = s->dl[e]; }
            else { a = k; b = s->di[e]; c = s->dj[e]; d = s->dl[e]; }
            v3 rb = mk(s->r[3 * b], s->r[3 * b + 1], s->r[3 * b + 2]);
            v3 b1 = minimg(sub(rb, mk(s->r[3 * a], s->r[3 * a + 1], s->r[3 * a + 2])), L);       /* a->b */
            v3 rc_ = mk(s->r[3 * c], s->r[3 * c + 1], s->r[3 * c + 2]);
            v3 b2 = minimg(sub(rc_, rb), L);                                                     /* b->c */
            v3 b3 = minimg(sub(mk(s->r[3 * d], s->r[3 * d + 1], s->r[3 * d + 2]), rc_), L);      /* c->d */
            v3 m = crs(b1, b2), nn = crs(b2, b3);
            double m2 = dot(m, m), n2 = dot(nn, nn), lb2 = nrm(b2);
            if(m2 < 1e-24 || n2 < 1e-24) continue;
            double cs = dot(m, nn) / sqrt(m2 * n2);
            if(cs > 1.0) cs = 1.0;
            if(cs < -1.0) cs = -1.0;
            double phi = acos(cs);                      /* standard unsigned dihedral */
            const double* p = s->dih_par + 4 * s->dt[e];
            int kind = s->dih_kind[s->dt[e]];
            double dV = dih_dU(kind, p, phi);
            double V = 0;
            if(kind == K_DIH_HARM) V = p[0] * (1.0 + (double)(int)p[1] * cos((double)(int)p[2] * phi));
            else if(kind == K_DIH_FOURIER4T)
                V = 0.5 * (p[0] * (1.0 + cos(phi)) + p[1] * (1.0 - cos(2.0 * phi)) + p[2] * (1.0 + cos(3.0 * phi)) + p[3] * (1.0 - cos(4.0 * phi)));
            /* gradients of the signed dihedral psi (|psi| = phi): standard Bekker/Blondel forms */
            v3 ga = scl(m, -lb2 / m2);
            v3 gd = scl(nn, lb2 / n2);
            double f1 = dot(b1, b2) / (lb2 * lb2), f3 = dot(b3, b2) / (lb2 * lb2);
            v3 gb = mk(-ga.x - f1 * ga.x + f3 * gd.x, -ga.y - f1 * ga.y + f3 * gd.y, -ga.z - f1 * ga.z + f3 * gd.z);
            /* sign of psi: s = sign(b1 . n) */
            double sgn = (dot(b1, nn) >= 0.0) ? 1.0 : -1.0;
            v3 g = s->dcen[e] ? gb : ga;
            fx -= dV * sgn * g.x; fy -= dV * sgn * g.y; fz -= dV * sgn * g.z;
            if(s->dcen[e]) uk += 0.5 * V;
            {
                /* r_k - r_X along a-b-c-d, X the lowest-index atom of the four */
                int X = a;
                if(b < X) X = b;
                if(c < X) X = c;
                if(d < X) X = d;
                v3 rel = mk(0.0, 0.0, 0.0);
                v3 r_a = mk(0.0, 0.0, 0.0), r_b = b1, r_c = mk(b1.x + b2.x, b1.y + b2.y, b1.z + b2.z);
                v3 r_d = mk(r_c.x + b3.x, r_c.y + b3.y, r_c.z + b3.z);   /* unwrapped chain from a */
                v3 rk_ = s->dcen[e] ? r_b : r_a;
                v3 rX = (X == a) ? r_a : (X == b) ? r_b : (X == c) ? r_c : r_d;
                rel = sub(rk_, rX);
                wk += -dV * sgn * dot(rel, g);
            }
        }
        /* non-bonded + Coulomb over all atoms (within cutoffs), in index order */
        const double qk = s->qd[k];
        for(int i = 0; i < s->n; i++) {
            if(i == k) continue;
            v3 d = minimg(sub(rk, mk(s->r[3 * i], s->r[3 * i + 1], s->r[3 * i + 2])), L);
            double R2 = dot(d, d), R = sqrt(R2);
            double md = 0.0, u = 0.0;
            if(R2 < rc2 && R >= 1e-3) {
                int pair = s->type[k] * T + s->type[i];
                for(int ff = 0; ff < s->nb_cnt[pair]; ff++) {
                    double m1, u1;
                    nb_analytic(s->nb_kind[pair * ORC_MAXFF + ff], s->nb_par + 4 * (pair * ORC_MAXFF + ff), R, rcut,
                                s->lj_shift, &m1, &u1);
                    md += m1; u += u1;
                }
            }
            double qi = s->qd[i];
            if(qk != 0.0 && qi != 0.0 && (s->coulomb_mode == 0 || R2 < crc2)) {
                double Kc = 1389.32 * qk * qi;
                if(s->coulomb_mode == 2) {       /* shifted force */
                    const double rq = s->coulomb_rc;
                    md += Kc * (1.0 / R2 - 1.0 / (rq * rq));
                    u += Kc * (1.0 / R - 1.0 / rq + (R - rq) / (rq * rq));
                } else {
                    md += Kc / R2;
                    u += Kc / R;
                }
            }
            if(md == 0.0 && u == 0.0) continue;
            int ap;
            float sc = exclusion_scale(s, k, i, &ap);
            double scd = ap ? (double)sc : 1.0;
            fx += scd * md * d.x / R; fy += scd * md * d.y / R; fz += scd * md * d.z / R;
            if(i > k) {
                uk += scd * u;
                wk += scd * md * R;
            }
        }
        F[3 * k] = fx; F[3 * k + 1] = fy; F[3 * k + 2] = fz;
        U[k] = uk;
        if(W) W[k] = wk;
    }
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* Reference-mode MD loop: MDLoop.cpp:128-133 with NVT (NH chain) or NVE, force clipping       */
/* ------------------------------------------------------------------------------------------ */
typedef struct orc_run {
    int ensemble;             /* 0 NVT, 1 NPT, 2 NVE */
    double dt;                /* reduced (fs / 100) */
    double kT;                /* NH_T_.T_ = T / Conv_T */
    double tau;               /* reduced */
    int M, nresp;             /* chain length, RESPA steps */
    double fcut;              /* cutoffforce; <= 0 disables clipping */
    int nx, ny, nz;           /* cell counts */
    /* NPT (SimulationBox.cpp:58-76): barostat chain NH_P_ and CVelVerlet W_, P_ */
    int MP, nrespP;           /* pressurenhlen, pressurerespa */
    double tauP;              /* reduced */
    double Pext;              /* pressure / Conv_press */
} orc_run;

static double cmt_exp(double x) { return (x > 1.0) ? 2.71828 * x : exp(x); }   /* Math.cpp:29-38 */

static double G0(const orc_sys* s, const double* p, double g, double beta) {
    double sum = 0.0;
    for(int k = 0; k < s->n; k++) {
        double p2 = p[3 * k] * p[3 * k] + p[3 * k + 1] * p[3 * k + 1] + p[3 * k + 2] * p[3 * k + 2];
        sum += (p2 / s->m[k]);
    }
    return sum - (g / beta);
}

/* CNHChain::propagator with CFctT (NHChain.cpp:54-113, MDLoop.cpp:29-60) */
static void nh_propagate(const orc_sys* s, const orc_run* c, double* p, double* eta, double* peta, const double* Q) {
    const double w0 = 1.0 / (1.0 - pow(2.0, 1.0 / 3.0));
    const double w[3] = {w0, 1.0 - 2.0 * w0, w0};
    const double beta = 1.0 / c->kT;
    const double g = (double)(3 * s->n);
    const int M = c->M;
    if(M > 0 && peta[0] > 15.0) peta[0] = 10.0;
#define GJ(j) ((j) == 0 ? G0(s, p, g, beta) : (peta[(j) - 1] * peta[(j) - 1] / Q[(j) - 1]) - (1.0 / beta))
    for(int mu = 0; mu < 3; mu++) {
        double Dt = w[mu] * c->dt / (double)c->nresp;
        for(int it = 0; it < c->nresp; it++) {
            peta[M - 1] += (Dt / 4.0) * GJ(M - 1);
            for(int j = 0; j < M - 1; j++) {
                double co = cmt_exp(-(Dt / 8.0) * (peta[j + 1] / Q[j + 1]));
                peta[j] *= co;
                peta[j] += (Dt / 4.0) * GJ(j);
                co = cmt_exp(-(Dt / 8.0) * (peta[j + 1] / Q[j + 1]));
                peta[j] *= co;
            }
            for(int j = 0; j < M; j++) eta[j] += (Dt / 2.0) * (peta[j] / Q[j]);
            double co = cmt_exp(-((Dt / 2.0) * (peta[0] / Q[0])));
            for(int k = 0; k < 3 * s->n; k++) p[k] *= co;
            for(int j = M - 2; j >= 0; j--) {
                double co2 = cmt_exp(-(Dt / 8.0) * (peta[j + 1] / Q[j + 1]));
                peta[j] *= co2;
                peta[j] += (Dt / 4.0) * GJ(j);
                co2 = cmt_exp(-(Dt / 8.0) * (peta[j + 1] / Q[j + 1]));
                peta[j] *= co2;
            }
            peta[M - 1] += (Dt / 4.0) * GJ(M - 1);
        }
    }
#undef GJ
}

/* CMt::sinhXoverX (Math.cpp:40-54): the first six terms of the Taylor series of sinh(x)/x. */
static double sinhx_over_x(double x) {
    const double a[6] = {1.0, 1.0 / 6.0, 1.0 / 120.0, 1.0 / 5040.0, 1.0 / 362880.0, 1.0 / 39916800.0};
    double sum = 0.0, xn = 1.0;
    for(int k = 0; k < 6; k++) {
        sum += a[k] * xn;
        xn *= (x * x);
    }
    return sum;
}

/* CNHChain::propagator with CFctP (NHChain.cpp:54-113, MDLoop.cpp:62-83): the barostat's chain,
 * G_0 = p_eps^2/W - kT, scaling p_eps. */
static void nhp_propagate(const orc_run* c, double* p_eps, double W, double* eta, double* peta, const double* Q) {
    const double w0 = 1.0 / (1.0 - pow(2.0, 1.0 / 3.0));
    const double w[3] = {w0, 1.0 - 2.0 * w0, w0};
    const double beta = 1.0 / c->kT;
    const int M = c->MP;
    if(M > 0 && peta[0] > 15.0) peta[0] = 10.0;
#define GP(j) ((j) == 0 ? (*p_eps) * (*p_eps) / W - (1.0 / beta) : (peta[(j) - 1] * peta[(j) - 1] / Q[(j) - 1]) - (1.0 / beta))
    for(int mu = 0; mu < 3; mu++) {
        double Dt = w[mu] * c->dt / (double)c->nrespP;
        for(int it = 0; it < c->nrespP; it++) {
            peta[M - 1] += (Dt / 4.0) * GP(M - 1);
            for(int j = 0; j < M - 1; j++) {
                double co = cmt_exp(-(Dt / 8.0) * (peta[j + 1] / Q[j + 1]));
                peta[j] *= co;
                peta[j] += (Dt / 4.0) * GP(j);
                co = cmt_exp(-(Dt / 8.0) * (peta[j + 1] / Q[j + 1]));
                peta[j] *= co;
            }
            for(int j = 0; j < M; j++) eta[j] += (Dt / 2.0) * (peta[j] / Q[j]);
            double co = cmt_exp(-((Dt / 2.0) * (peta[0] / Q[0])));
            *p_eps *= co;
            for(int j = M - 2; j >= 0; j--) {
                double co2 = cmt_exp(-(Dt / 8.0) * (peta[j + 1] / Q[j + 1]));
                peta[j] *= co2;
                peta[j] += (Dt / 4.0) * GP(j);
                co2 = cmt_exp(-(Dt / 8.0) * (peta[j + 1] / Q[j + 1]));
                peta[j] *= co2;
            }
            peta[M - 1] += (Dt / 4.0) * GP(M - 1);
        }
    }
#undef GP
}

/* CVelVerlet::G_eps (VelVerlet.cpp:160-174) */
static double g_eps(const orc_sys* s, const double* p, const double* F, const double* r, double V, double Pext) {
    double sum_p = 0.0, sum_f = 0.0;
    for(int k = 0; k < s->n; k++) {
        double p2 = p[3 * k] * p[3 * k] + p[3 * k + 1] * p[3 * k + 1] + p[3 * k + 2] * p[3 * k + 2];
        sum_p += (p2 / s->m[k]);
        sum_f += (F[3 * k] * r[3 * k] + F[3 * k + 1] * r[3 * k + 1] + F[3 * k + 2] * r[3 * k + 2]);
    }
    return (1.0 + 1.0 / (double)s->n) * sum_p + sum_f - 3.0 * Pext * V;
}

/* CVelVerlet::prop_p (VelVerlet.cpp:124-136) */
static void prop_p(const orc_sys* s, double dt, double p_eps, double W, double* p, const double* F) {
    double u_eps = p_eps / W;
    double alpha = (1.0 + 1.0 / (double)s->n);
    double parm = alpha * u_eps * dt / 4.0;
    double coeff = cmt_exp(-parm);
    double coeff2 = coeff * coeff;
    double coeff3 = sinhx_over_x(parm);
    double b = (dt / 2.0) * coeff * coeff3;
    for(int k = 0; k < 3 * s->n; k++) p[k] = p[k] * coeff2 + F[k] * b;
}

/* CVelVerlet::prop_r (VelVerlet.cpp:138-150) */
static void prop_r(const orc_sys* s, double dt, double p_eps, double W, double* r, const double* p) {
    double u_eps = p_eps / W;
    double parm = u_eps * dt / 2.0;
    double coeff = cmt_exp(parm);
    double coeff2 = coeff * coeff;
    double coeff3 = sinhx_over_x(parm) * coeff;
    double b = dt * coeff3;
    for(int k = 0; k < s->n; k++) {
        double im = 1.0 / s->m[k];
        for(int a = 0; a < 3; a++) r[3 * k + a] = r[3 * k + a] * coeff2 + (p[3 * k + a] * im) * b;
    }
}

typedef struct orc_lists {
    int* atom_cell; int* cell_ptr; int* cell_list; int* count; int* list; int maxn;
} orc_lists;

static int ref_forces(orc_sys* s, const orc_run* c, orc_lists* ls, double* F, float* U) {
    const float Lf[3] = {(float)s->box[0], (float)s->box[1], (float)s->box[2]};
    orc_cell_list(s->n, s->r, Lf, c->nx, c->ny, c->nz, ls->atom_cell, ls->cell_ptr, ls->cell_list);
    int need = orc_neigh_list(s->n, s->r, Lf, s->rc, c->nx, c->ny, c->nz, ls->atom_cell, ls->cell_ptr, ls->cell_list,
                              ls->maxn, ls->count, ls->list);
    if(need > ls->maxn) {
        free(ls->list);
        ls->maxn = need + 10;
        ls->list = (int*)malloc((size_t)s->n * ls->maxn * sizeof(int));
        if(!ls->list) return -1;
        orc_neigh_list(s->n, s->r, Lf, s->rc, c->nx, c->ny, c->nz, ls->atom_cell, ls->cell_ptr, ls->cell_list,
                       ls->maxn, ls->count, ls->list);
    }
    return orc_forces_ref(s, ls->count, ls->list, ls->maxn, F, U);
}

/* Runs nsteps.  r, p (n*3), eta, peta (M) are updated in place, and for NPT also
 * baro = [p_eps, eps, eta_P[MP], p_eta_P[MP]] (the box follows eps, VelVerlet.cpp:198-211).  Every `stride` steps (and at the
 * start) it records r, p, F into rec_* ([nrec][n][3]) and U, K, T, P, V into rec_scal ([nrec][5]).
 * Returns the number of records or a negative error. */
int orc_run_ref(orc_sys* s, const orc_run* c, double* r, double* p, double* eta, double* peta, double* baro,
                int nsteps, int stride, double* rec_r, double* rec_p, double* rec_F, double* rec_scal) {
    const int n = s->n;
    double* F = (double*)calloc((size_t)3 * n, sizeof(double));
    float* U = (float*)calloc((size_t)n, sizeof(float));
    double* Q = (double*)calloc((size_t)(c->M > 0 ? c->M : 1), sizeof(double));
    orc_lists ls;
    ls.atom_cell = (int*)malloc((size_t)3 * n * sizeof(int));
    ls.cell_ptr = (int*)malloc((size_t)2 * c->nx * c->ny * c->nz * sizeof(int));
    ls.cell_list = (int*)malloc((size_t)n * sizeof(int));
    ls.count = (int*)malloc((size_t)n * sizeof(int));
    ls.maxn = 10;
    ls.list = (int*)malloc((size_t)n * ls.maxn * sizeof(int));
    s->r = r;
    Q[0] = (double)(3 * n) * c->kT * c->tau * c->tau;
    for(int j = 1; j < c->M; j++) Q[j] = c->kT * c->tau * c->tau;
    double V = s->box[0] * s->box[1] * s->box[2];
    /* NPT state: baro = [p_eps, eps, eta_P[MP], p_eta_P[MP]] (VelVerlet.h:57-62, NH_P_) */
    const int npt = (c->ensemble == 1);
    const double Lmax[3] = {s->box[0], s->box[1], s->box[2]};
    const double V0 = Lmax[0] * Lmax[1] * Lmax[2];
    const double W = c->kT * c->tauP * c->tauP;
    double QP[64];
    if(npt) {
        if(c->MP < 1 || c->MP > 64) return -2;
        QP[0] = 1.0 * c->kT * c->tauP * c->tauP;    /* prepareArrays(1, 1): dim*N = 1 */
        for(int j = 1; j < c->MP; j++) QP[j] = c->kT * c->tauP * c->tauP;
    }
    int nrec = 0;
    int rc_ = ref_forces(s, c, &ls, F, U);
    if(rc_ < 0) return rc_;
    for(int t = -1; t < nsteps; t++) {
        if(t >= 0 && npt) {
            /* MDLoop.cpp:128-133 with VelVerlet.cpp:57-71 (no force clipping in this branch) */
            double* p_eps = &baro[0];
            double* eps = &baro[1];
            double* etaP = baro + 2;
            double* petaP = baro + 2 + c->MP;
            nhp_propagate(c, p_eps, W, etaP, petaP, QP);
            nh_propagate(s, c, p, eta, peta, Q);
            V = V0 * exp(3.0 * (*eps));
            *p_eps += ((c->dt / 2.0) * g_eps(s, p, F, r, V, c->Pext));     /* 3.1 */
            prop_p(s, c->dt, *p_eps, W, p, F);                             /* 3.2 */
            prop_r(s, c->dt, *p_eps, W, r, p);                             /* 3.3 */
            *eps += (c->dt * (*p_eps) / W);                                /* 3.4 */
            {
                /* getSimBox (VelVerlet.cpp:198-211) */
                double Vmax = Lmax[0] * Lmax[1] * Lmax[2];
                double etaCube = (V0 * exp(3.0 * (*eps))) / Vmax;
                etaCube = pow(etaCube, 1.0 / 3.0);
                for(int a = 0; a < 3; a++) s->box[a] = etaCube * Lmax[a];
            }
            rc_ = ref_forces(s, c, &ls, F, U);
            if(rc_ < 0) return rc_;
            prop_p(s, c->dt, *p_eps, W, p, F);                             /* 3.5 */
            V = V0 * exp(3.0 * (*eps));
            *p_eps += ((c->dt / 2.0) * g_eps(s, p, F, r, V, c->Pext));     /* 3.6 */
            nh_propagate(s, c, p, eta, peta, Q);
            nhp_propagate(c, p_eps, W, etaP, petaP, QP);
            for(int k = 0; k < n; k++) {
                for(int a = 0; a < 3; a++) {
                    double Lm = s->box[a], h = Lm / 2.0;
                    double* x = &r[3 * k + a];
                    if(*x >= h) *x -= (double)((int)((*x + h) / Lm)) * Lm;
                    if(*x < -h) *x -= (double)((int)((*x + (-h)) / Lm)) * Lm;
                }
            }
        } else if(t >= 0) {
            if(c->ensemble == 0) nh_propagate(s, c, p, eta, peta, Q);
            double dt_2 = c->dt / 2.0;
            for(int k = 0; k < n; k++) {
                double m_k = s->m[k];
                for(int a = 0; a < 3; a++) p[3 * k + a] += F[3 * k + a] * dt_2;
                double dm = c->dt / m_k;
                for(int a = 0; a < 3; a++) r[3 * k + a] += p[3 * k + a] * dm;
            }
            rc_ = ref_forces(s, c, &ls, F, U);
            if(rc_ < 0) return rc_;
            if(c->fcut > 0) {
                for(int k = 0; k < 3 * n; k++) {
                    if(fabs(F[k]) > c->fcut) F[k] = ((F[k] >= 0.0) ? 1.0 : -1.0) * c->fcut;
                }
            }
            for(int k = 0; k < 3 * n; k++) p[k] += F[k] * dt_2;
            if(c->ensemble == 0) nh_propagate(s, c, p, eta, peta, Q);
            /* pbcWrap (SimulationBox.cpp:135-166) */
            for(int k = 0; k < n; k++) {
                for(int a = 0; a < 3; a++) {
                    double Lm = s->box[a], h = Lm / 2.0;
                    double* x = &r[3 * k + a];
                    if(*x >= h) *x -= (double)((int)((*x + h) / Lm)) * Lm;
                    if(*x < -h) *x -= (double)((int)((*x + (-h)) / Lm)) * Lm;
                }
            }
        }
        if(t == -1 || ((t + 1) % stride) == 0 || t == nsteps - 1) {
            double Ut = 0.0, K2 = 0.0, Ps = 0.0;
            for(int k = 0; k < n; k++) Ut += (double)U[k];
            for(int k = 0; k < n; k++) {
                double p2 = (p[3 * k] * p[3 * k] + p[3 * k + 1] * p[3 * k + 1] + p[3 * k + 2] * p[3 * k + 2]) / s->m[k];
                K2 += p2;
                double fr = F[3 * k] * r[3 * k] + F[3 * k + 1] * r[3 * k + 1] + F[3 * k + 2] * r[3 * k + 2];
                Ps += (p2 + fr);
            }
            if(rec_r) memcpy(rec_r + (size_t)nrec * 3 * n, r, (size_t)3 * n * sizeof(double));
            if(rec_p) memcpy(rec_p + (size_t)nrec * 3 * n, p, (size_t)3 * n * sizeof(double));
            if(rec_F) memcpy(rec_F + (size_t)nrec * 3 * n, F, (size_t)3 * n * sizeof(double));
            if(rec_scal) {
                double* o = rec_scal + (size_t)nrec * 5;
                o[0] = Ut; o[1] = 0.5 * K2; o[2] = K2 / (3.0 * (double)n); o[3] = (1.0 / (3.0 * V)) * Ps; o[4] = V;
            }
            nrec++;
        }
    }
    if(npt) for(int a = 0; a < 3; a++) s->box[a] = Lmax[a];
    free(F); free(U); free(Q);
    free(ls.atom_cell); free(ls.cell_ptr); free(ls.cell_list); free(ls.count); free(ls.list);
    return nrec;
}
