// Initial momenta and thermostat / barostat state (host side).  Compiled without fused
// multiply-adds so the reference mode's numbers are the same on x86-64 and aarch64 hosts.
//
// MTG_INIT_REFERENCE reproduces what CSimulationBox::initSystem draws (SimulationBox.cpp:53-96):
//   NH_T_.setRandNHPos, NH_P_.setRandNHPos (NHChain.cpp:126-133), setRandMom
//   (SimulationBox.cpp:98-133), NH_T_.setRandNHMom, NH_P_.setRandNHMom (NHChain.cpp:135-143),
//   velVerlet_.setRandMom (VelVerlet.cpp:176-182)
// from the C library's rand() seeded with `seed` (a fresh process behaves as seed 1; the reference
// draws in the CSimulationBox constructor, before CMDLoop::runSimulation calls srand(time),
// MDLoop.cpp:118).  setRandMom scales the momenta to T before copyPosFromState has copied the
// masses in, so the scaling uses the particles' default mass of 1 g/mol (Particle3D.cpp:25-27);
// that is reproduced, not corrected.
//
// MTG_INIT_MAXWELL draws Maxwell-Boltzmann momenta (mass-correct, centre-of-mass momentum of the
// mobile atoms removed, rescaled so that sum p^2/m / 3N = kT, the reference's temperature
// estimator), chain positions uniform in [0, 1) and thermal chain and barostat momenta
// N(0, Q kT), N(0, W kT), from a seeded SplitMix64 stream with Box-Muller normals.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "mtg_internal.h"

namespace mtg {
namespace {

// The C library's rand() (the additive feedback generator of degree 31 and separation 3 behind
// random(): a Lehmer seeding of the 31-word table, 310 discarded outputs, then
// r[i] = r[i-3] + r[i-31] mod 2^32 and the output r[i] >> 1), RAND_MAX = 2^31 - 1.
class LibcRand {
public:
    explicit LibcRand(uint32_t seed) {
        int32_t w = seed == 0 ? 1 : (int32_t)seed;
        t_[0] = (uint32_t)w;
        for(int i = 1; i < 31; i++) {
            // 16807 w mod (2^31 - 1) without overflow (Schrage's method)
            const int32_t hi = w / 127773, lo = w % 127773;
            w = 16807 * lo - 2836 * hi;
            if(w < 0) w += 2147483647;
            t_[i] = (uint32_t)w;
        }
        f_ = 3;
        r_ = 0;
        for(int i = 0; i < 310; i++) next();
    }
    int32_t next() {
        t_[f_] += t_[r_];
        const int32_t out = (int32_t)(t_[f_] >> 1);
        f_ = (f_ + 1) % 31;
        r_ = (r_ + 1) % 31;
        return out;
    }

private:
    uint32_t t_[31];
    int f_, r_;
};

constexpr double kRandMax = 2147483647.0;

struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }   // [0, 1)
    double normal() {
        double u = uniform();
        while(u <= 0.0) u = uniform();
        const double v = uniform();
        return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
    }
};

}  // namespace

int draw_initial_state(int n, const double* mass, const uint8_t* mobile, const mtg_config_desc* cfg, uint32_t seed,
                       int mode, double* p, mtg_thermo_state* th) {
    const double kT = cfg->temperature / kConvT;               // NH_T_.T_ = NH_P_.T_
    const double tauT = cfg->temperature_relax / kConvt;
    const double tauP = cfg->pressure_relax / kConvt;
    const int M = cfg->temperature_nh_len, MP = cfg->pressure_nh_len;
    if(n <= 0 || M < 0 || MP < 0 || M > kMaxChain || MP > kMaxChain) return MTG_E_INVALID;
    std::vector<double> QT(std::max(M, 1)), QP(std::max(MP, 1));
    for(int j = 0; j < M; j++) QT[j] = (j == 0 ? double(3 * n) : 1.0) * kT * tauT * tauT;   // prepareArrays(N, 3)
    for(int j = 0; j < MP; j++) QP[j] = (j == 0 ? 1.0 : 1.0) * kT * tauP * tauP;            // prepareArrays(1, 1)
    const double W = kT * tauP * tauP;
    std::memset(th, 0, sizeof(*th));
    th->M = M;
    th->MP = MP;
    const auto is_mobile = [&](int k) { return mobile ? mobile[k] != 0 : true; };
    if(mode == MTG_INIT_REFERENCE) {
        LibcRand rnd(seed);
        const double a = 2.0 / kRandMax;
        for(int j = 0; j < M; j++) th->eta[j] = double(rnd.next()) / kRandMax;
        for(int j = 0; j < MP; j++) th->etaP[j] = double(rnd.next()) / kRandMax;
        for(int k = 0; k < n; k++) {
            for(int a3 = 0; a3 < 3; a3++) {
                double v = a * double(rnd.next()) - 1.0;
                p[3 * k + a3] = v;
            }
            for(int a3 = 0; a3 < 3; a3++)
                if(p[3 * k + a3] == 0.0) p[3 * k + a3] = 1.0;
        }
        for(int k = 0; k < n; k++)
            if(!is_mobile(k)) p[3 * k] = p[3 * k + 1] = p[3 * k + 2] = 0.0;
        // calcTemp with the default particle mass of 1 (the masses are copied in afterwards)
        double T = 0.0;
        for(int k = 0; k < n; k++) {
            const double pp = p[3 * k] * p[3 * k] + p[3 * k + 1] * p[3 * k + 1] + p[3 * k + 2] * p[3 * k + 2];
            T += pp / 1.0;
        }
        const double Tnow = T / (3 * double(n));
        const double s = std::sqrt(kT / Tnow);
        for(int k = 0; k < 3 * n; k++) p[k] *= s;
        for(int j = 0; j < M; j++) {
            th->p_eta[j] = (a * double(rnd.next()) - 1.0) * (QT[j] / tauT);
            if(th->p_eta[j] == 0.0) th->p_eta[j] = QT[j] / tauT;
        }
        for(int j = 0; j < MP; j++) {
            th->p_etaP[j] = (a * double(rnd.next()) - 1.0) * (QP[j] / tauP);
            if(th->p_etaP[j] == 0.0) th->p_etaP[j] = QP[j] / tauP;
        }
        th->p_eps = (a * double(rnd.next()) - 1.0) * (W / tauP);
        if(th->p_eps == 0.0) th->p_eps = W / tauP;
        return MTG_OK;
    }
    if(mode != MTG_INIT_MAXWELL) return MTG_E_INVALID;
    SplitMix rnd{0x6D74675F696E6974ull ^ (uint64_t)seed};
    int nmob = 0;
    double com[3] = {0.0, 0.0, 0.0};
    for(int k = 0; k < n; k++) {
        if(!is_mobile(k)) {
            p[3 * k] = p[3 * k + 1] = p[3 * k + 2] = 0.0;
            continue;
        }
        const double sd = std::sqrt(mass[k] * kT);
        for(int a3 = 0; a3 < 3; a3++) {
            p[3 * k + a3] = sd * rnd.normal();
            com[a3] += p[3 * k + a3];
        }
        nmob++;
    }
    if(nmob > 1)
        for(int k = 0; k < n; k++)
            if(is_mobile(k))
                for(int a3 = 0; a3 < 3; a3++) p[3 * k + a3] -= com[a3] / nmob;
    double T = 0.0;
    for(int k = 0; k < n; k++)
        T += (p[3 * k] * p[3 * k] + p[3 * k + 1] * p[3 * k + 1] + p[3 * k + 2] * p[3 * k + 2]) / mass[k];
    const double Tnow = T / (3.0 * n);
    if(Tnow > 0.0) {
        const double s = std::sqrt(kT / Tnow);
        for(int k = 0; k < 3 * n; k++) p[k] *= s;
    }
    for(int j = 0; j < M; j++) th->eta[j] = rnd.uniform();
    for(int j = 0; j < M; j++) th->p_eta[j] = std::sqrt(QT[j] * kT) * rnd.normal();
    for(int j = 0; j < MP; j++) th->etaP[j] = rnd.uniform();
    for(int j = 0; j < MP; j++) th->p_etaP[j] = std::sqrt(QP[j] * kT) * rnd.normal();
    th->p_eps = std::sqrt(W * kT) * rnd.normal();
    return MTG_OK;
}

}  // namespace mtg
