// Oracle harness (test infrastructure only; never part of the product path).
//
// Project-written driver that replaces the reference's src/main.cpp:11-37 so the
// unmodified reference hot path can be run as an oracle:
//   Parser(config)                      -> src/Parser.cpp:13-23
//   nbgrp::init()                       -> src/NBGroup.cpp:129-139
//   optional initial state / seeded noise written into nbgrp::nmr::nubm_0
//     (the loop recomputes S(psi0) at its start, src/Nmr.cpp:117-121)
//   nbgrp::nmr::evolutionLoop()         -> src/Nmr.cpp:89-262
// and then writes the accepted-step log, the final state and (optionally) the
// intermediate stage buffers and the per-step tables to raw files.
//
// usage: xflat_ref_{ma,maa,sa} <config> [--state-in F] [--noise SEED AMP]
//            [--state-out F] [--log F] [--stages PREFIX] [--probe F]
//
// File formats: raw little-endian float64.  States use the reference's NetCDF
// psi layout [beam][comp(ar,ai,br,bi)][ebin] (src/IO_f.cpp:280-288).
// --probe writes a sequence of records {char name[32]; int64 n; double v[n]}.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <time.h>
#include <stdint.h>

#include "global.h"
#include "Parser.h"
#include "Util.h"
#include "NBGroup.h"
#include "Nmr.h"
#include "NBeam.h"
#include "Matt.h"
#include "Phy.h"

namespace oracle_io {
extern std::vector<double> accepted;
extern const nbm::NBeam* last_state;
extern long n_accepted;
}

namespace nbgrp {
namespace nmr {
extern nbm::NBeam* nubm_0;
extern nbm::NBeam* nubm_1;
extern nbm::NBeam* nubm_3;
extern nbm::NBeam* nubm_4;
}
#if defined(MAA)
namespace phy_maa {
extern double* L_E;
extern double* cos_tetbins;
extern double* sin_tetbins;
extern double* dcos_tetbins;
extern double* delta_l;
extern int tetbins;
}
#elif defined(SA)
namespace phy_sa {
extern double* L_E;
extern double* rarr;
extern double* delta_l;
}
#else
namespace phy_ma {
extern double* L_E;
extern double* cos_tbin;
extern double* dcos_tbin;
extern double* delta_l;
extern int tetbins;
}
#endif
}
namespace nbm { extern double* h_vacc; }

// Counter-based noise generator shared (as a specification) with the GPU host
// code and the C restatement: splitmix64 keyed on (seed, beam, ebin, k).
static uint64_t sm64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ULL;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static double noise_u01(uint64_t seed, uint64_t beam, uint64_t e, uint64_t k)
{
    uint64_t h = sm64(seed ^ sm64((beam << 24) ^ (e << 1) ^ k));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

static void write_raw(const char* path, const std::vector<double>& v)
{
    FILE* f = fopen(path, "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", path); exit(2); }
    if (!v.empty()) fwrite(v.data(), sizeof(double), v.size(), f);
    fclose(f);
}

static std::vector<double> gather_state(const nbm::NBeam* b, int len, int ne)
{
    std::vector<double> out((size_t)len * 4 * ne);
    for (int i = 0; i < len; ++i)
        for (int c = 0; c < 4; ++c)
            memcpy(&out[((size_t)i * 4 + c) * ne], b[i].psi(c), ne * sizeof(double));
    return out;
}

static void probe_rec(FILE* f, const char* name, const double* v, int64_t n)
{
    char nm[32];
    memset(nm, 0, sizeof nm);
    strncpy(nm, name, 31);
    fwrite(nm, 1, 32, f);
    fwrite(&n, sizeof n, 1, f);
    fwrite(v, sizeof(double), (size_t)n, f);
}

int main(int argc, char* argv[])
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s <config> [options]\n", argv[0]);
        return 2;
    }
    const char *state_in = 0, *state_out = 0, *log_out = 0, *stages = 0, *probe = 0;
    uint64_t seed = 0;
    double amp = 0.;
    bool noise = false;
    for (int i = 2; i < argc; ++i) {
        std::string a = argv[i];
        if (a == "--state-in" && i + 1 < argc) state_in = argv[++i];
        else if (a == "--state-out" && i + 1 < argc) state_out = argv[++i];
        else if (a == "--log" && i + 1 < argc) log_out = argv[++i];
        else if (a == "--stages" && i + 1 < argc) stages = argv[++i];
        else if (a == "--probe" && i + 1 < argc) probe = argv[++i];
        else if (a == "--noise" && i + 2 < argc) {
            seed = strtoull(argv[i + 1], 0, 10);
            amp = atof(argv[i + 2]);
            noise = true;
            i += 2;
        } else {
            fprintf(stderr, "unknown option %s\n", argv[i]);
            return 2;
        }
    }

    Parser parser(argv[1]);
    Util::inVals(NULL);
    nbgrp::init();

    const int len = nbgrp::phy::beamLen();
    const int ne = nbm::nbm_ebins;
    nbm::NBeam* b0 = nbgrp::nmr::nubm_0;

    if (state_in) {
        FILE* f = fopen(state_in, "rb");
        if (!f) { fprintf(stderr, "cannot read %s\n", state_in); return 2; }
        std::vector<double> buf((size_t)len * 4 * ne);
        size_t got = fread(buf.data(), sizeof(double), buf.size(), f);
        fclose(f);
        if (got != buf.size()) { fprintf(stderr, "short state file\n"); return 2; }
        for (int i = 0; i < len; ++i)
            for (int c = 0; c < 4; ++c)
                memcpy(b0[i].psi(c), &buf[((size_t)i * 4 + c) * ne], ne * sizeof(double));
    } else if (noise) {
        for (int i = 0; i < len; ++i) {
            const int p = i % 4;
            for (int e = 0; e < ne; ++e) {
                double eps = (noise_u01(seed, i, e, 0) - 0.5) * amp;
                double eta = (noise_u01(seed, i, e, 1) - 0.5) * amp;
                double one_sq = sqrt(1. - eps * eps - eta * eta);
                b0[i].Ar(e) = (p < 2) ? one_sq : eps;
                b0[i].Ai(e) = 0.;
                b0[i].Br(e) = (p < 2) ? eps : one_sq;
                b0[i].Bi(e) = eta;
            }
        }
    }

    if (probe) {
        // Tables and one Hamiltonian evaluation per stage point on the initial state.
        FILE* f = fopen(probe, "wb");
        if (!f) { fprintf(stderr, "cannot write %s\n", probe); return 2; }
        std::vector<double> fv(4 * ne);
        for (int p = 0; p < 4; ++p)
            for (int e = 0; e < ne; ++e) fv[p * ne + e] = b0[p].Fv(e);
        probe_rec(f, "fv", fv.data(), fv.size());
        probe_rec(f, "hvac", nbm::h_vacc, 2 * ne);
        double ev[4] = {nbm::Ev(0), nbm::Ev(1), nbm::Ev(2), nbm::Ev(3)};
        probe_rec(f, "Ev", ev, 4);
        const double r = Util::R0(), dr = Util::dr();
        const double dr2 = .5 * dr, rdr = r + dr, rdr2 = r + dr2;
        double hm[3];
        matt::getHm(r, hm[0]);
        matt::getHm(rdr2, hm[1]);
        matt::getHm(rdr, hm[2]);
        probe_rec(f, "hm", hm, 3);
        nbgrp::phy::calcAngleBins(r, 0);
        nbgrp::phy::calcAngleBins(rdr2, 1);
        nbgrp::phy::calcAngleBins(rdr, 2);
        nbgrp::phy::calcDeltaLs(dr2, 0, 0, 1);
        nbgrp::phy::calcDeltaLs(dr, 1, 0, 2);
        nbgrp::phy::calcDeltaLs(dr2, 2, 1, 2);
#if defined(MAA)
        namespace P = nbgrp::phy_maa;
        probe_rec(f, "LE", P::L_E, 4);
        probe_rec(f, "cos", P::cos_tetbins, 3 * P::tetbins);
        probe_rec(f, "sin", P::sin_tetbins, 3 * P::tetbins);
        probe_rec(f, "dcos", P::dcos_tetbins, 3 * P::tetbins);
        probe_rec(f, "dl", P::delta_l, 3 * P::tetbins);
        const int nh = len;  // (theta*phi) * 4 doubles = len
#elif defined(SA)
        namespace P = nbgrp::phy_sa;
        probe_rec(f, "LE", P::L_E, 4);
        probe_rec(f, "rpt", P::rarr, 3);
        probe_rec(f, "dl", P::delta_l, 3);
        const int nh = 4;  // one 4-vector shared by the four particle beams
#else
        namespace P = nbgrp::phy_ma;
        probe_rec(f, "LE", P::L_E, 4);
        probe_rec(f, "cos", P::cos_tbin, 3 * P::tetbins);
        probe_rec(f, "dcos", P::dcos_tbin, 3 * P::tetbins);
        probe_rec(f, "dl", P::delta_l, 3 * P::tetbins);
        const int nh = len;  // theta * 4 doubles = len
#endif
        for (int i = 0; i < len; ++i) b0[i].calcESum();
        std::vector<double> hs(4 * (size_t)len);
        for (int i = 0; i < len; ++i) b0[i].getESum(&hs[4 * (size_t)i]);
        probe_rec(f, "esum0", hs.data(), hs.size());
        double* hvv;
        nbgrp::phy::newHvv(hvv);
        for (int pt = 0; pt < 3; ++pt) {
            nbgrp::phy::calc_Hvv(b0, pt, hvv);
            char nm[16];
            snprintf(nm, sizeof nm, "hvv%d", pt);
            probe_rec(f, nm, hvv, nh);
        }
        nbgrp::phy::deleteHvv(hvv);
        fclose(f);
    }

    timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int iters = nbgrp::nmr::evolutionLoop();
    clock_gettime(CLOCK_MONOTONIC, &t1);
    double secs = (t1.tv_sec - t0.tv_sec) + 1e-9 * (t1.tv_nsec - t0.tv_nsec);

    const nbm::NBeam* fin = oracle_io::last_state ? oracle_io::last_state : b0;
    if (state_out) write_raw(state_out, gather_state(fin, len, ne));
    if (log_out) write_raw(log_out, oracle_io::accepted);
    if (stages) {
        std::string pre = stages;
        write_raw((pre + "_psi0.bin").c_str(), gather_state(nbgrp::nmr::nubm_0, len, ne));
        write_raw((pre + "_psi1.bin").c_str(), gather_state(nbgrp::nmr::nubm_1, len, ne));
        write_raw((pre + "_psi3.bin").c_str(), gather_state(nbgrp::nmr::nubm_3, len, ne));
        write_raw((pre + "_psi4.bin").c_str(), gather_state(nbgrp::nmr::nubm_4, len, ne));
        std::vector<double> hs(4 * (size_t)len), errs(len);
        for (int i = 0; i < len; ++i) nbgrp::nmr::nubm_4[i].getESum(&hs[4 * (size_t)i]);
        write_raw((pre + "_esum4.bin").c_str(), hs);
        for (int i = 0; i < len; ++i) errs[i] = nbgrp::nmr::nubm_4[i].calcErrHvv(nbgrp::nmr::nubm_1[i]);
        write_raw((pre + "_err.bin").c_str(), errs);
    }
    printf("{\"iterations\": %d, \"accepted\": %ld, \"seconds\": %.6f, \"beams\": %d, \"ebins\": %d}\n",
           iters, oracle_io::n_accepted, secs, len, ne);
    nbgrp::freemem();
    return 0;
}
