// 1000-point force/potential tables of the MDFF terms, generated on the host.
//
// The reference builds these in CMDFFMatrices::prepareFFMatrices (MDFFMatrices.cpp:263-382) by
// calling each term's calc1DForceProfile / calc1DPotentialProfile (MolTwisterMDFFNonBonded.cpp:126-172,
// MolTwisterMDFFBond.cpp:133-179, MolTwisterMDFFAngle.cpp:210-257, MolTwisterMDFFDih.cpp:272-320).
// A table point is (x, F_x / (dx/dx_x), U): the force on the last atom of a probe geometry divided by
// the matching geometry coefficient, i.e. -dU/dx up to rounding.  The drop-in path receives the
// tables from the MDFF classes themselves; this generator serves callers that pass only term
// parameters.  It evaluates every expression in the reference's order and is compiled without
// fused multiply-adds, so its tables are bit-identical to the reference's (checked by the tests).
#include <cmath>

#include "mtg_internal.h"

namespace mtg {
namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dotp(V3 a, V3 b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); }
inline double length(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double safe_inv(double R) { return (R == 0.0) ? 1.0 / 1E-10 : 1.0 / R; }

// d r / d r2 for r = |r2 - r1| (calcNonBondForceCoeffs12 / calcBondForceCoeffs12)
V3 unit12(V3 r1, V3 r2) {
    V3 d = r2 - r1;
    return d * safe_inv(length(d));
}

// d theta / d r3 for the angle r1-r2-r3 (calcAngularForceCoeffs13)
V3 angle_coeff13(V3 r1, V3 r2, V3 r3) {
    V3 K = (r1 - r2) * safe_inv(length(r1 - r2));
    V3 u = r3 - r2;
    double A = K.x * u.x + K.y * u.y + K.z * u.z;
    double B = u.x * u.x + u.y * u.y + u.z * u.z;
    double sB = std::sqrt(B);
    double sB3 = (B == 0.0) ? std::sqrt(1E-30) : sB * sB * sB;
    double gx = (K.x * B - u.x * A) / sB3, gy = (K.y * B - u.y * A) / sB3, gz = (K.z * B - u.z * A) / sB3;
    double W = (sB == 0.0) ? A / 10E-3 : A / sB;
    double den = std::sqrt(1.0 - W * W);
    double f = (den == 0.0) ? -1.0 / 1E-10 : -1.0 / den;
    return {f * gx, f * gy, f * gz};
}

// d phi / d r4 for the dihedral r1-r2-r3-r4 (calcDihedralForceCoeffs14)
V3 dihedral_coeff14(V3 r1, V3 r2, V3 r3, V3 r4) {
    V3 r21 = r1 - r2, r23 = r3 - r2;
    V3 r32 = r23 * (-1.0);
    V3 r34 = r4 - r3;
    V3 n1 = cross(r23, r21);
    V3 K = n1 * safe_inv(length(n1));
    double a = r32.y * r34.z - r32.z * r34.y;
    double b = r32.z * r34.x - r32.x * r34.z;
    double c = r32.x * r34.y - r32.y * r34.x;
    double A = K.x * a + K.y * b + K.z * c;
    double B = a * a + b * b + c * c;
    double sBi = (B == 0.0) ? 1.0 / 1E-20 : 1.0 / std::sqrt(B);
    double sBi3 = sBi * sBi * sBi;
    double W = A * sBi;
    double gx = ((K.y * r32.z - K.z * r32.y) * B - (r32.z * (r32.z * r34.x - r32.x * r34.z) - r32.y * (r32.x * r34.y - r32.y * r34.x)) * A) * sBi3;
    double gy = ((K.z * r32.x - K.x * r32.z) * B - (r32.x * (r32.x * r34.y - r32.y * r34.x) - r32.z * (r32.y * r34.z - r32.z * r34.y)) * A) * sBi3;
    double gz = ((K.x * r32.y - K.y * r32.x) * B - (r32.y * (r32.y * r34.z - r32.z * r34.y) - r32.x * (r32.z * r34.x - r32.x * r34.z)) * A) * sBi3;
    double den = std::sqrt(1.0 - W * W);
    double f = (den == 0.0) ? 1.0 / 1E-10 : 1.0 / den;
    V3 o = {f * gx, f * gy, f * gz};
    return o * (-1.0);
}

// Pair terms: force component on r2 along x, and the potential.
double pair_force_x(int kind, const double* p, V3 r1, V3 r2) {
    V3 d = r2 - r1;
    double R = length(d);
    double Ri = safe_inv(R);
    double Ri2 = Ri * Ri;
    double g;
    switch(kind) {
    case MTG_NB_LJ: {
        double Ri6 = Ri2 * Ri2 * Ri2, Ri12 = Ri6 * Ri6;
        double s2 = p[1] * p[1], s6 = s2 * s2 * s2, s12 = s6 * s6;
        g = 4.0 * p[0] * Ri2 * (12.0 * s12 * Ri12 - 6.0 * p[2] * s6 * Ri6);
        break;
    }
    case MTG_NB_LJ1208: {
        double Ri4 = Ri2 * Ri2, Ri6 = Ri4 * Ri2, Ri8 = Ri4 * Ri4, Ri12 = Ri6 * Ri6;
        double s2 = p[1] * p[1], s4 = s2 * s2, s6 = s4 * s2, s8 = s4 * s4, s12 = s6 * s6;
        g = 4.0 * p[0] * Ri2 * (12.0 * s12 * Ri12 - 8.0 * p[2] * s8 * Ri8);
        break;
    }
    case MTG_NB_BUCK: {
        double Ri4 = Ri2 * Ri2, Ri6 = Ri4 * Ri2;
        double rhoi = (p[1] == 0.0) ? 1E-10 : 1.0 / p[1];
        g = Ri2 * (p[0] * R * rhoi * std::exp(-R * rhoi) - 6.0 * p[2] * Ri6);
        break;
    }
    default:
        return 0.0;
    }
    return d.x * g;
}

double pair_potential(int kind, const double* p, V3 r1, V3 r2) {
    double R = length(r2 - r1);
    double Ri = safe_inv(R);
    double Ri2 = Ri * Ri;
    switch(kind) {
    case MTG_NB_LJ: {
        double Ri6 = Ri2 * Ri2 * Ri2, Ri12 = Ri6 * Ri6;
        double s2 = p[1] * p[1], s6 = s2 * s2 * s2, s12 = s6 * s6;
        return 4.0 * p[0] * (s12 * Ri12 - p[2] * s6 * Ri6);
    }
    case MTG_NB_LJ1208: {
        double Ri4 = Ri2 * Ri2, Ri6 = Ri4 * Ri2, Ri8 = Ri4 * Ri4, Ri12 = Ri6 * Ri6;
        double s2 = p[1] * p[1], s4 = s2 * s2, s6 = s4 * s2, s8 = s4 * s4, s12 = s6 * s6;
        (void)Ri6;
        return 4.0 * p[0] * (s12 * Ri12 - p[2] * s8 * Ri8);
    }
    case MTG_NB_BUCK: {
        double Ri4 = Ri2 * Ri2, Ri6 = Ri4 * Ri2;
        double rhoi = (p[1] == 0.0) ? 1E-10 : 1.0 / p[1];
        return p[0] * std::exp(-R * rhoi) - p[2] * Ri6;
    }
    default:
        return 0.0;
    }
}

double bond_force_x(int kind, const double* p, V3 r1, V3 r2) {
    V3 d = r2 - r1;
    double R = length(d);
    double Ri = safe_inv(R);
    double g;
    if(kind == MTG_BOND_HARM) {
        double dR = R - p[1];
        g = -2.0 * p[0] * dR * Ri;
    } else if(kind == MTG_BOND_MORSE) {
        double dR = R - p[2];
        double e = std::exp(-p[1] * dR);
        g = -2.0 * p[0] * p[1] * Ri * e * (1.0 - e);
    } else {
        return 0.0;
    }
    return d.x * g;
}

double bond_potential(int kind, const double* p, V3 r1, V3 r2) {
    double R = length(r2 - r1);
    if(kind == MTG_BOND_HARM) {
        double dR = R - p[1];
        return p[0] * dR * dR;
    }
    if(kind == MTG_BOND_MORSE) {
        double dR = R - p[2];
        double q = (1.0 - std::exp(-p[1] * dR));
        return p[0] * q * q;
    }
    return 0.0;
}

double angle_value(V3 r1, V3 r2, V3 r3) {
    V3 a = r1 - r2, b = r3 - r2;
    double ia = safe_inv(length(a)), ib = safe_inv(length(b));
    return std::acos(dotp(a, b) * (ia * ib));
}

double dihedral_value(V3 r1, V3 r2, V3 r3, V3 r4) {
    V3 r21 = r1 - r2, r23 = r3 - r2;
    V3 r32 = r23 * (-1.0);
    V3 r34 = r4 - r3;
    V3 n1 = cross(r23, r21), n2 = cross(r32, r34);
    double nn = length(n1) * length(n2);
    double c = (nn == 0.0) ? dotp(n1, n2) / 1E-20 : dotp(n1, n2) / nn;
    return std::acos(c);
}

double dihedral_dU(int kind, const double* p, double phi) {
    if(kind == MTG_DIH_HARM) {
        int D = (int)p[1], N = (int)p[2];
        return -p[0] * double(D * N) * std::sin(double(N) * phi);
    }
    if(kind == MTG_DIH_FOURIER4T) {
        double a = -0.5 * p[0] * std::sin(phi);
        double b = p[1] * std::sin(2.0 * phi);
        double c = -1.5 * p[2] * std::sin(3.0 * phi);
        double d = 2.0 * p[3] * std::sin(4.0 * phi);
        return a + b + c + d;
    }
    return 0.0;
}

double dihedral_U(int kind, const double* p, double phi) {
    if(kind == MTG_DIH_HARM) return p[0] * (1.0 + double((int)p[1]) * std::cos(double((int)p[2]) * phi));
    if(kind == MTG_DIH_FOURIER4T) {
        double u1 = p[0] * (1.0 + std::cos(phi)), u2 = p[1] * (1.0 - std::cos(2.0 * phi));
        double u3 = p[2] * (1.0 + std::cos(3.0 * phi)), u4 = p[3] * (1.0 - std::cos(4.0 * phi));
        return 0.5 * (u1 + u2 + u3 + u4);
    }
    return 0.0;
}

inline float ratio(double f, double c) { return (float)((c != 0.0) ? f / c : 0.0); }

}  // namespace

int profile_nonbonded(int kind, const double* p, float r0, float r1, int npts, float* out) {
    if(kind != MTG_NB_LJ && kind != MTG_NB_LJ1208 && kind != MTG_NB_BUCK) return MTG_E_UNSUPPORTED;
    float step = (r1 - r0) / float(npts - 1);
    for(int i = 0; i < npts; i++) {
        float r = r0 + float(i) * step;
        V3 a{0, 0, 0}, b{double(r), 0, 0};
        out[3 * i] = r;
        out[3 * i + 1] = ratio(pair_force_x(kind, p, a, b), unit12(a, b).x);
        out[3 * i + 2] = (float)pair_potential(kind, p, a, b);
    }
    return MTG_OK;
}

int profile_bond(int kind, const double* p, float r0, float r1, int npts, float* out) {
    if(kind != MTG_BOND_HARM && kind != MTG_BOND_MORSE && kind != MTG_BOND_LJC) return MTG_E_UNSUPPORTED;
    float step = (r1 - r0) / float(npts - 1);
    for(int i = 0; i < npts; i++) {
        float r = r0 + float(i) * step;
        V3 a{0, 0, 0}, b{double(r), 0, 0};
        out[3 * i] = r;
        out[3 * i + 1] = ratio(bond_force_x(kind, p, a, b), unit12(a, b).x);
        out[3 * i + 2] = (float)bond_potential(kind, p, a, b);
    }
    return MTG_OK;
}

int profile_angle(int kind, const double* p, float t0, float t1, int npts, float* out) {
    if(kind != MTG_ANGLE_HARM) return MTG_E_UNSUPPORTED;
    float step = (t1 - t0) / float(npts - 1);
    for(int i = 0; i < npts; i++) {
        float t = t0 + float(i) * step;
        V3 a{-1.0, 0, 0}, b{0, 0, 0}, c{-std::cos(double(t)), std::sin(double(t)), 0.0};
        double dt = angle_value(a, b, c) - p[1] * p[2];
        V3 g = angle_coeff13(a, b, c);
        out[3 * i] = t;
        out[3 * i + 1] = ratio(g.x * (-2.0 * p[0] * dt), g.x);
        out[3 * i + 2] = (float)(p[0] * dt * dt);
    }
    return MTG_OK;
}

int profile_dihedral(int kind, const double* p, float t0, float t1, int npts, float* out) {
    if(kind != MTG_DIH_HARM && kind != MTG_DIH_FOURIER4T) return MTG_E_UNSUPPORTED;
    float step = (t1 - t0) / float(npts - 1);
    for(int i = 0; i < npts; i++) {
        float t = t0 + float(i) * step;
        V3 a{0, 1.0, 0}, b{0, 0, 0}, c{0, 0, 1.0}, d{std::sin(double(t)), std::cos(double(t)), 1.0};
        double phi = dihedral_value(a, b, c, d);
        V3 g = dihedral_coeff14(a, b, c, d);
        out[3 * i] = t;
        out[3 * i + 1] = ratio(g.x * dihedral_dU(kind, p, phi), g.x);
        out[3 * i + 2] = (float)dihedral_U(kind, p, phi);
    }
    return MTG_OK;
}

}  // namespace mtg
