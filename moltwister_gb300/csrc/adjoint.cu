// Adjoint (reverse-mode) kernels for parameter gradients of energies and of short-trajectory
// losses: tangents of the analytic forces in FP64 forward-mode dual numbers (positions or
// force-field coefficients carry the tangent), the Gaussian-smeared pair correlation of two atom
// types and its position gradient, and the small vector kernels of the backward recursion.
//
// The force expressions follow the production kernels (md_kernels.cu) term by term: 12-6 / 12-8
// LJ and Buckingham with per-term cutoffs and energy shifts, cut-off and shifted-force Coulomb,
// harmonic / Morse bonds, harmonic angles, harmonic / Fourier4t dihedrals, exclusion scaling by
// neighbour-list class.  Tabulated kinds have no derivative and are rejected by the host.
#include <cuda_runtime.h>
#include <stdint.h>

#include "md_device.cuh"
#include "mtg_internal.h"

namespace mtg {
namespace {

// ---------------------------------------------------------------------------------------------
// Forward-mode dual numbers: v + t eps, eps^2 = 0
// ---------------------------------------------------------------------------------------------
struct Dual {
    double v, t;
    __device__ Dual() : v(0.0), t(0.0) {}
    __device__ Dual(double x) : v(x), t(0.0) {}
    __device__ Dual(double x, double dx) : v(x), t(dx) {}
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.t + b.t); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.t - b.t); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.t); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.t * b.v + a.v * b.t); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double iv = 1.0 / b.v;
    return Dual(a.v * iv, (a.t - a.v * iv * b.t) * iv);
}
__device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) { a = a + b; return a; }
__device__ __forceinline__ Dual& operator-=(Dual& a, Dual b) { a = a - b; return a; }
__device__ __forceinline__ Dual& operator*=(Dual& a, Dual b) { a = a * b; return a; }
__device__ __forceinline__ Dual dsqrt(Dual a) {
    const double s = sqrt(a.v);
    return Dual(s, a.t * 0.5 / s);
}
__device__ __forceinline__ Dual dexp(Dual a) {
    const double e = exp(a.v);
    return Dual(e, a.t * e);
}
__device__ __forceinline__ Dual dsin(Dual a) { return Dual(sin(a.v), a.t * cos(a.v)); }
__device__ __forceinline__ Dual dcos(Dual a) { return Dual(cos(a.v), -a.t * sin(a.v)); }
// acos on [-1, 1]; the derivative is taken with sin(theta) >= 1e-6, as the force kernels clamp it
__device__ __forceinline__ Dual dacos(Dual a) {
    const double c = a.v > 1.0 ? 1.0 : (a.v < -1.0 ? -1.0 : a.v);
    double s = sqrt(1.0 - c * c);
    s = s < 1e-6 ? 1e-6 : s;
    return Dual(acos(c), -a.t / s);
}

struct D3 {
    Dual x, y, z;
};
__device__ __forceinline__ Dual dot(const D3& a, const D3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 cross(const D3& a, const D3& b) {
    return D3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Tangent inputs: positions (vpos, 3n) and/or coefficient tables and charges.
struct Tangents {
    const double* vpos;      // [3n] position tangents, or null
    const double* nb_par_t;  // [T*T*5*4] tangents of the non-bonded coefficients, or null
    const double* nb_fs_t;   // [T*T*5] tangents of the LJ force at the cutoff, or null
    const double* q_t;       // [n] charge tangents, or null
    const double* bond_par_t;
    const double* angle_par_t;
    const double* dih_par_t;
};

__device__ __forceinline__ Dual tdual(double v, const double* t, int k) { return Dual(v, t ? t[k] : 0.0); }

// Minimum-image separation r_i - r_j of the system atom i belongs to, with the tangent
// v_i - v_j (wrapping moves an atom by a box vector, which carries no tangent).
__device__ __forceinline__ D3 rel_d(const DevSys& d, const Params& P, const double* pos, int i, int j, const double* vpos) {
    double L[3];
    if(P.nrep) {
        const RepDev& R = d.reps[d.rep_of[i]];
        L[0] = R.box[0]; L[1] = R.box[1]; L[2] = R.box[2];
    } else {
        L[0] = P.box[0]; L[1] = P.box[1]; L[2] = P.box[2];
    }
    D3 o;
    Dual* c[3] = {&o.x, &o.y, &o.z};
    for(int a = 0; a < 3; a++) {
        const double dd = minimg_d(pos[3 * i + a] - pos[3 * j + a], L[a], 1.0 / L[a]);
        *c[a] = Dual(dd, vpos ? vpos[3 * i + a] - vpos[3 * j + a] : 0.0);
    }
    return o;
}

// Pair force on i from j (g * d, g = -dU/dr / r) and pair energy, in dual numbers.
__device__ void pair_dual(const DevSys& d, const Params& P, const Tangents& tg, int i, int j, int cls, const D3& dv,
                          float rc, float rcoul, D3& f, Dual& u) {
    f = D3{};
    u = Dual(0.0);
    const Dual r2 = dot(dv, dv);
    if(r2.v < 1e-6) return;
    const Dual r = dsqrt(r2);
    const Dual ir = Dual(1.0) / r;
    const Dual ir2 = ir * ir;
    Dual g(0.0);
    if(r2.v < double(rc) * double(rc)) {
        const int pr = d.type[i] * P.T + d.type[j];
        for(int ff = 0; ff < d.nb_cnt[pr]; ff++) {
            const int idx = pr * kMaxFF + ff;
            const int kind = d.nb_kind[idx];
            const Dual a = tdual(d.nb_par[4 * idx], tg.nb_par_t, 4 * idx);
            const Dual b = tdual(d.nb_par[4 * idx + 1], tg.nb_par_t, 4 * idx + 1);
            const Dual c = tdual(d.nb_par[4 * idx + 2], tg.nb_par_t, 4 * idx + 2);
            const Dual dd = tdual(d.nb_par[4 * idx + 3], tg.nb_par_t, 4 * idx + 3);
            if(kind == MTG_NB_LJ || kind == MTG_NB_LJ1208) {
                if(c.v == 0.0 || r2.v < c.v) {
                    const Dual ir6 = ir2 * ir2 * ir2;
                    const Dual irn = kind == MTG_NB_LJ ? ir6 : ir6 * ir2;
                    const double nn = kind == MTG_NB_LJ ? 6.0 : 8.0;
                    const Dual t12 = a * ir6 * ir6, tn = b * irn;
                    g += (Dual(12.0) * t12 - Dual(nn) * tn) * ir2;
                    u += t12 - tn - dd;
                    if(P.lj_shift == 2) {
                        const Dual fs = tdual(d.nb_fs[idx], tg.nb_fs_t, idx);
                        g -= fs * ir;
                        u += r * fs;
                    }
                }
            } else if(kind == MTG_NB_BUCK) {
                const Dual ir6 = ir2 * ir2 * ir2;
                const Dual e = a * dexp(-(r * b));
                g += e * b * ir - Dual(6.0) * c * ir6 * ir2;
                u += e - c * ir6;
            }
        }
    }
    if(P.coulomb != MTG_COULOMB_ALLPAIRS && r2.v < double(rcoul) * double(rcoul)) {
        const Dual qi = tdual(d.qd[i], tg.q_t, i), qj = tdual(d.qd[j], tg.q_t, j);
        const Dual qq = Dual(1389.32) * qi * qj;
        const double irc = 1.0 / double(rcoul);
        if(P.coulomb == MTG_COULOMB_SHIFTED) {
            g += qq * (ir2 - Dual(irc * irc)) * ir;
            u += qq * (ir - Dual(irc) + (r - Dual(double(rcoul))) * Dual(irc * irc));
        } else {
            g += qq * ir2 * ir;
            u += qq * ir;
        }
    }
    if(cls) {
        const Dual sc((double)P.scale[cls]);
        g *= sc;
        u *= sc;
    }
    f = D3{g * dv.x, g * dv.y, g * dv.z};
}

// Bonded entry e of atom k (bonds, angles, dihedrals of k, as bonded_entry in md_kernels.cu).
__device__ void bonded_dual(const DevSys& d, const Params& P, const Tangents& tg, const double* pos, int k, int e, D3& f,
                            Dual& u) {
    const int nb = d.bptr[k + 1] - d.bptr[k];
    const int na = d.aptr[k + 1] - d.aptr[k];
    if(e < nb) {
        const int q = d.bptr[k] + e;
        const int i = d.bj[q], t = d.bt[q];
        const D3 dv = rel_d(d, P, pos, k, i, tg.vpos);     // r_k - r_i
        const Dual r = dsqrt(dot(dv, dv));
        const Dual p0 = tdual(d.bond_par[4 * t], tg.bond_par_t, 4 * t);
        const Dual p1 = tdual(d.bond_par[4 * t + 1], tg.bond_par_t, 4 * t + 1);
        const Dual p2 = tdual(d.bond_par[4 * t + 2], tg.bond_par_t, 4 * t + 2);
        Dual md(0.0), uu(0.0);
        if(d.bond_kind[t] == MTG_BOND_HARM) {
            const Dual dr = r - p1;
            md = Dual(-2.0) * p0 * dr;
            uu = p0 * dr * dr;
        } else if(d.bond_kind[t] == MTG_BOND_MORSE) {
            const Dual ex = dexp(-(p1 * (r - p2)));
            md = Dual(-2.0) * p0 * p1 * ex * (Dual(1.0) - ex);
            uu = p0 * (Dual(1.0) - ex) * (Dual(1.0) - ex);
        }
        const Dual s = md / r;
        f.x += s * dv.x; f.y += s * dv.y; f.z += s * dv.z;
        if(i > k) u += uu;
        return;
    }
    e -= nb;
    if(e < na) {
        const int q = d.aptr[k] + e;
        const int t = d.at[q];
        int c, a1, a3;
        if(d.acen[q]) { c = k; a1 = d.ai[q]; a3 = d.aj[q]; }
        else { c = d.ai[q]; a1 = k; a3 = d.aj[q]; }
        const D3 uv = rel_d(d, P, pos, a1, c, tg.vpos);
        const D3 vv = rel_d(d, P, pos, a3, c, tg.vpos);
        const Dual n1 = dsqrt(dot(uv, uv)), n3 = dsqrt(dot(vv, vv));
        const Dual cs = dot(uv, vv) / (n1 * n3);
        const Dual th = dacos(cs);
        Dual sn = dsqrt(Dual(1.0) - cs * cs);
        if(sn.v < 1e-6) sn = Dual(1e-6);
        const Dual kk = tdual(d.angle_par[4 * t], tg.angle_par_t, 4 * t);
        const Dual t0 = tdual(d.angle_par[4 * t + 1], tg.angle_par_t, 4 * t + 1);
        const Dual dd = th - t0;
        const Dual dU = Dual(2.0) * kk * dd;
        const Dual uu = kk * dd * dd;
        const Dual inv = Dual(1.0) / (n1 * n3);
        const Dual i1 = cs / (n1 * n1), i3 = cs / (n3 * n3);
        const D3 g1{-(vv.x * inv - i1 * uv.x) / sn, -(vv.y * inv - i1 * uv.y) / sn, -(vv.z * inv - i1 * uv.z) / sn};
        if(d.acen[q]) {
            const D3 g3{-(uv.x * inv - i3 * vv.x) / sn, -(uv.y * inv - i3 * vv.y) / sn, -(uv.z * inv - i3 * vv.z) / sn};
            f.x += dU * (g1.x + g3.x); f.y += dU * (g1.y + g3.y); f.z += dU * (g1.z + g3.z);
            u += uu;
        } else {
            f.x -= dU * g1.x; f.y -= dU * g1.y; f.z -= dU * g1.z;
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
        const D3 b1 = rel_d(d, P, pos, b, a, tg.vpos);
        const D3 b2 = rel_d(d, P, pos, c, b, tg.vpos);
        const D3 b3 = rel_d(d, P, pos, dd, c, tg.vpos);
        const D3 m = cross(b1, b2), nn = cross(b2, b3);
        const Dual m2 = dot(m, m), n2 = dot(nn, nn);
        if(!(m2.v > 1e-20 && n2.v > 1e-20)) return;
        const Dual lb2 = dsqrt(dot(b2, b2));
        const Dual cs = dot(m, nn) / dsqrt(m2 * n2);
        const Dual phi = dacos(cs);
        const Dual p0 = tdual(d.dih_par[4 * t], tg.dih_par_t, 4 * t);
        const Dual p1 = tdual(d.dih_par[4 * t + 1], tg.dih_par_t, 4 * t + 1);
        const Dual p2 = tdual(d.dih_par[4 * t + 2], tg.dih_par_t, 4 * t + 2);
        const Dual p3 = tdual(d.dih_par[4 * t + 3], tg.dih_par_t, 4 * t + 3);
        Dual dV(0.0), V(0.0);
        if(d.dih_kind[t] == MTG_DIH_HARM) {
            const int D = (int)d.dih_par[4 * t + 1], N = (int)d.dih_par[4 * t + 2];
            dV = -(p0 * Dual(double(D * N)) * dsin(Dual(double(N)) * phi));
            V = p0 * (Dual(1.0) + Dual(double(D)) * dcos(Dual(double(N)) * phi));
        } else if(d.dih_kind[t] == MTG_DIH_FOURIER4T) {
            dV = Dual(-0.5) * p0 * dsin(phi) + p1 * dsin(Dual(2.0) * phi) + Dual(-1.5) * p2 * dsin(Dual(3.0) * phi) +
                 Dual(2.0) * p3 * dsin(Dual(4.0) * phi);
            V = Dual(0.5) * (p0 * (Dual(1.0) + dcos(phi)) + p1 * (Dual(1.0) - dcos(Dual(2.0) * phi)) +
                             p2 * (Dual(1.0) + dcos(Dual(3.0) * phi)) + p3 * (Dual(1.0) - dcos(Dual(4.0) * phi)));
        }
        const double sgn = dot(b1, nn).v >= 0.0 ? 1.0 : -1.0;
        const Dual ga = -(lb2 / m2), gd = lb2 / n2;
        D3 gv;
        if(d.dcen[q]) {
            const Dual f1 = dot(b1, b2) / (lb2 * lb2), f3 = dot(b3, b2) / (lb2 * lb2);
            const Dual cm = -(Dual(1.0) + f1) * ga, cn = f3 * gd;
            gv = D3{cm * m.x + cn * nn.x, cm * m.y + cn * nn.y, cm * m.z + cn * nn.z};
            u += Dual(0.5) * V;
        } else {
            gv = D3{ga * m.x, ga * m.y, ga * m.z};
        }
        const Dual s = dV * Dual(sgn);
        f.x -= s * gv.x; f.y -= s * gv.y; f.z -= s * gv.z;
    }
}

// Force and energy tangents of every atom (one warp per atom over its Verlet-list row, then its
// bonded entries): Ft[3i..] = d F_i, Ut[i] = d U_i (the reference's per-atom energy bookkeeping).
__global__ void k_force_tangent(DevSys d, Params P, const double* pos, Tangents tg, double* Ft, double* Ut) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if(i >= P.n) return;
    double fx = 0.0, fy = 0.0, fz = 0.0, uu = 0.0;
    if(d.mobile[i]) {
        float rc = P.rc, rq = P.rcoul;
        if(P.nrep) {
            const RepDev& R = d.reps[d.rep_of[i]];
            rc = R.rc;
            rq = R.rcoul;
        }
        const int si = d.slot_of[i];   // list rows and entries are slots (cell order)
        const int cnt = min(d.vcount[si], d.vmax);
        const uint32_t* lst = d.vlist + (size_t)si * d.vmax;
        for(int e = lane; e < cnt; e += 32) {
            const uint32_t ent = lst[e];
            const int j = d.pcell_list[ent & kIdxMask], cls = (int)(ent >> kClassShift);
            const D3 dv = rel_d(d, P, pos, i, j, tg.vpos);
            D3 f;
            Dual u;
            pair_dual(d, P, tg, i, j, cls, dv, rc, rq, f, u);
            fx += f.x.t; fy += f.y.t; fz += f.z.t;
            if(j > i) uu += u.t;
        }
        const int nbd = (d.bptr[i + 1] - d.bptr[i]) + (d.aptr[i + 1] - d.aptr[i]) + (d.dptr[i + 1] - d.dptr[i]);
        for(int b = lane; b < nbd; b += 32) {
            D3 f{};
            Dual u(0.0);
            bonded_dual(d, P, tg, pos, i, b, f, u);
            fx += f.x.t; fy += f.y.t; fz += f.z.t;
            uu += u.t;
        }
    }
    for(int o = 16; o > 0; o >>= 1) {
        fx += __shfl_down_sync(0xffffffffu, fx, o);
        fy += __shfl_down_sync(0xffffffffu, fy, o);
        fz += __shfl_down_sync(0xffffffffu, fz, o);
        uu += __shfl_down_sync(0xffffffffu, uu, o);
    }
    if(lane == 0) {
        Ft[3 * i] = fx;
        Ft[3 * i + 1] = fy;
        Ft[3 * i + 2] = fz;
        if(Ut) Ut[i] = uu;
    }
}

// ---------------------------------------------------------------------------------------------
// Gaussian-smeared pair correlation between atom types ta and tb
// ---------------------------------------------------------------------------------------------
// Each pair contributes to the bins whose centre lies within kWin widths of r (the Gaussian there
// is e^-32 = 1e-14 of its peak, so the truncation leaves the loss smooth to rounding).
constexpr double kWin = 8.0;

struct RdfSpec {
    int ta, tb, nbins;
    double rmax, width, dr;
};

// Row i of the smeared histogram: sum over list partners j (type tb; j > i when ta == tb) of
// K(r_ij - x_b), K the unit-area Gaussian of the given width, x_b = (b + 1/2) dr, |r - x_b| <= kWin w.  Lane l owns
// bins b = l, l + 32, ..., so every bin is summed in list order by one lane (deterministic).
__global__ void k_rdf_rows(DevSys d, Params P, const double* pos, RdfSpec s, double* rows) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if(i >= P.n) return;
    double* row = rows + (size_t)i * s.nbins;
    for(int b = lane; b < s.nbins; b += 32) row[b] = 0.0;
    const int ti = d.type[i];
    if(ti != s.ta && ti != s.tb) return;
    const double iw2 = 1.0 / (s.width * s.width), norm = 1.0 / (s.width * 2.5066282746310002);
    const int si = d.slot_of[i];
    const int cnt = min(d.vcount[si], d.vmax);
    const uint32_t* lst = d.vlist + (size_t)si * d.vmax;
    for(int e = 0; e < cnt; e++) {
        const int j = d.pcell_list[lst[e] & kIdxMask];
        const int tj = d.type[j];
        const bool pair = (s.ta == s.tb) ? (ti == s.ta && tj == s.tb && j > i) : (ti == s.ta && tj == s.tb);
        if(!pair) continue;
        const D3 dv = rel_d(d, P, pos, i, j, nullptr);
        const double r = sqrt(dot(dv, dv).v);
        if(r > s.rmax + kWin * s.width) continue;
        const int b0 = max(0, (int)floor((r - kWin * s.width) / s.dr)), b1 = min(s.nbins - 1, (int)floor((r + kWin * s.width) / s.dr));
        for(int b = b0 + lane; b <= b1; b += 32) {
            const double x = r - (b + 0.5) * s.dr;
            if(fabs(x) <= kWin * s.width) row[b] += norm * exp(-0.5 * x * x * iw2);
        }
    }
}

// hist[b] += sum over rows (fixed row order)
__global__ void k_rdf_reduce(const double* rows, int n, int nbins, double* hist) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if(b >= nbins) return;
    double s = 0.0;
    for(int i = 0; i < n; i++) s += rows[(size_t)i * nbins + b];
    hist[b] += s;
}

// grad_i += sum_b c_b d/dr_i K(r_ij - x_b) over the pairs atom i belongs to (gather over its row)
__global__ void k_rdf_adjoint(DevSys d, Params P, const double* pos, RdfSpec s, const double* cb, double* grad) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if(i >= P.n) return;
    const int ti = d.type[i];
    if(ti != s.ta && ti != s.tb) return;
    const double iw2 = 1.0 / (s.width * s.width), norm = 1.0 / (s.width * 2.5066282746310002);
    double gx = 0.0, gy = 0.0, gz = 0.0;
    const int si = d.slot_of[i];
    const int cnt = min(d.vcount[si], d.vmax);
    const uint32_t* lst = d.vlist + (size_t)si * d.vmax;
    for(int e = 0; e < cnt; e++) {
        const int j = d.pcell_list[lst[e] & kIdxMask];
        const int tj = d.type[j];
        const bool pair = (ti == s.ta && tj == s.tb) || (ti == s.tb && tj == s.ta);
        if(!pair) continue;
        const D3 dv = rel_d(d, P, pos, i, j, nullptr);
        const double r = sqrt(dot(dv, dv).v);
        if(r > s.rmax + kWin * s.width || r < 1e-9) continue;
        const int b0 = max(0, (int)floor((r - kWin * s.width) / s.dr)), b1 = min(s.nbins - 1, (int)floor((r + kWin * s.width) / s.dr));
        double dk = 0.0;
        for(int b = b0 + lane; b <= b1; b += 32) {
            const double x = r - (b + 0.5) * s.dr;
            if(fabs(x) <= kWin * s.width) dk += cb[b] * (-x * iw2) * norm * exp(-0.5 * x * x * iw2);
        }
        const double ir = 1.0 / r;
        gx += dk * dv.x.v * ir;
        gy += dk * dv.y.v * ir;
        gz += dk * dv.z.v * ir;
    }
    for(int o = 16; o > 0; o >>= 1) {
        gx += __shfl_down_sync(0xffffffffu, gx, o);
        gy += __shfl_down_sync(0xffffffffu, gy, o);
        gz += __shfl_down_sync(0xffffffffu, gz, o);
    }
    if(lane == 0) {
        grad[3 * i] += gx;
        grad[3 * i + 1] += gy;
        grad[3 * i + 2] += gz;
    }
}

// ---------------------------------------------------------------------------------------------
// Vector kernels of the backward recursion
// ---------------------------------------------------------------------------------------------
// y[k] += a * x[k] * (per-atom scale s[k/3] when s != null)
__global__ void k_axpy(int n3, double a, const double* x, const double* s, double* y) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k >= n3) return;
    y[k] += a * x[k] * (s ? s[k / 3] : 1.0);
}

// out[blockIdx.x] = sum over the block's range of x[k] * y[k] (y null: sum of x), fixed order
__global__ void k_dot_blocks(int n, const double* x, const double* y, double* out) {
    __shared__ double smem[32];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {k < n ? x[k] * (y ? y[k] : 1.0) : 0.0};
    block_sum<1>(v, smem);
    if(threadIdx.x == 0) out[blockIdx.x] = v[0];
}

// out[0] += w * sum of nb partials (fixed order, one thread)
__global__ void k_accum_partials(const double* part, int nb, double w, double* out) {
    if(threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for(int b = 0; b < nb; b++) s += part[b];
    out[0] += w * s;
}

// out[s] = sum of x[off[s] .. off[s+1]) in a fixed order (one block per segment: strided thread
// sums, then the fixed shuffle tree of block_sum): per-replica totals of a batch.
__global__ void k_segment_sums(const double* x, const int* off, double* out) {
    __shared__ double smem[32];
    const int a = off[blockIdx.x], b = off[blockIdx.x + 1];
    double v[1] = {0.0};
    for(int k = a + (int)threadIdx.x; k < b; k += blockDim.x) v[0] += x[k];
    block_sum<1>(v, smem);
    if(threadIdx.x == 0) out[blockIdx.x] = v[0];
}

__global__ void k_inv_mass(int n, const double* m, double* im) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if(k < n) im[k] = 1.0 / m[k];
}

// Pair-distance histogram of CCmdPairCorrelation::execute for one frame
// (Cmd/MolTwisterCmdCalculate/CmdPairCorrelation.cpp:182-215): every ordered pair (i in A, j in B),
// distance across the periodic box as C3DVector::distToAcrossPBC (Utilities/3DVector.cpp:44-66),
// pairs closer than ignore_below skipped, bin int((R - rmin) / (rmax - rmin) * nbins).  The
// arithmetic is spelled out with round-to-nearest intrinsics so no contraction changes a bin.
__global__ void k_pair_hist(const double* pos, const int* ia, int na, const int* ib, int nb, double wx, double wy, double wz,
                            double rmin, double rmax, int nbins, double ignore_below, unsigned long long* prof) {
    extern __shared__ unsigned int hist_s[];
    for(int b = threadIdx.x; b < nbins; b += blockDim.x) hist_s[b] = 0u;
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if(t < na) {
        const int i = ia[t];
        const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
        const double span = __dsub_rn(rmax, rmin);
        for(int q = 0; q < nb; q++) {
            const int j = ib[q];
            double dX = __dsub_rn(xi, pos[3 * j]), dY = __dsub_rn(yi, pos[3 * j + 1]), dZ = __dsub_rn(zi, pos[3 * j + 2]);
            dX = (dX < 0.0) ? -dX : dX;
            dY = (dY < 0.0) ? -dY : dY;
            dZ = (dZ < 0.0) ? -dZ : dZ;
            if(dX > wx / 2.0) dX = __dsub_rn(wx, dX);
            if(dY > wy / 2.0) dY = __dsub_rn(wy, dY);
            if(dZ > wz / 2.0) dZ = __dsub_rn(wz, dZ);
            const double R = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dX, dX), __dmul_rn(dY, dY)), __dmul_rn(dZ, dZ)));
            if(R < ignore_below) continue;
            const int n = (int)__dmul_rn(__ddiv_rn(__dsub_rn(R, rmin), span), double(nbins));
            if(n >= 0 && n < nbins) atomicAdd(&hist_s[n], 1u);
        }
    }
    __syncthreads();
    for(int b = threadIdx.x; b < nbins; b += blockDim.x)
        if(hist_s[b]) atomicAdd(&prof[b], (unsigned long long)hist_s[b]);
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

void launch_pair_hist(const double* pos, const int* ia, int na, const int* ib, int nb, const double* box, double rmin,
                      double rmax, int nbins, double ignore_below, unsigned long long* prof, cudaStream_t s) {
    k_pair_hist<<<nblk(na, 128), 128, sizeof(unsigned int) * nbins, s>>>(pos, ia, na, ib, nb, box[0], box[1], box[2], rmin,
                                                                        rmax, nbins, ignore_below, prof);
}

// ---------------------------------------------------------------------------------------------
// Launchers (declared in mtg_internal.h)
// ---------------------------------------------------------------------------------------------
void launch_force_tangent(const DevSys& d, const Params& P, const double* pos, const AdjTangents& t, double* Ft, double* Ut,
                          cudaStream_t s) {
    Tangents tg{t.vpos, t.nb_par_t, t.nb_fs_t, t.q_t, t.bond_par_t, t.angle_par_t, t.dih_par_t};
    k_force_tangent<<<nblk((long long)P.n * 32, 128), 128, 0, s>>>(d, P, pos, tg, Ft, Ut);
}

void launch_rdf_rows(const DevSys& d, const Params& P, const double* pos, const AdjRdf& r, double* rows, cudaStream_t s) {
    RdfSpec sp{r.ta, r.tb, r.nbins, r.rmax, r.width, r.rmax / r.nbins};
    k_rdf_rows<<<nblk((long long)P.n * 32, 128), 128, 0, s>>>(d, P, pos, sp, rows);
}

void launch_rdf_reduce(const double* rows, int n, int nbins, double* hist, cudaStream_t s) {
    k_rdf_reduce<<<nblk(nbins, 128), 128, 0, s>>>(rows, n, nbins, hist);
}

void launch_rdf_adjoint(const DevSys& d, const Params& P, const double* pos, const AdjRdf& r, const double* cb, double* grad,
                        cudaStream_t s) {
    RdfSpec sp{r.ta, r.tb, r.nbins, r.rmax, r.width, r.rmax / r.nbins};
    k_rdf_adjoint<<<nblk((long long)P.n * 32, 128), 128, 0, s>>>(d, P, pos, sp, cb, grad);
}

void launch_axpy(int n3, double a, const double* x, const double* scale, double* y, cudaStream_t s) {
    k_axpy<<<nblk(n3, 256), 256, 0, s>>>(n3, a, x, scale, y);
}

int dot_blocks(int n) { return nblk(n, 256); }

void launch_dot_blocks(int n, const double* x, const double* y, double* out, cudaStream_t s) {
    k_dot_blocks<<<nblk(n, 256), 256, 0, s>>>(n, x, y, out);
}

void launch_segment_sums(const double* x, const int* off, int nseg, double* out, cudaStream_t s) {
    k_segment_sums<<<nseg, 256, 0, s>>>(x, off, out);
}

void launch_inv_mass(int n, const double* m, double* im, cudaStream_t s) { k_inv_mass<<<nblk(n, 256), 256, 0, s>>>(n, m, im); }

void launch_dot_accum(int n, const double* x, const double* y, double w, double* part, double* out, cudaStream_t s) {
    const int nb = nblk(n, 256);
    k_dot_blocks<<<nb, 256, 0, s>>>(n, x, y, part);
    k_accum_partials<<<1, 32, 0, s>>>(part, nb, w, out);
}

}  // namespace mtg
