// Host-side physics set-up (see xf_physics.h).
#include "xf_physics.h"

#include <algorithm>
#include <cmath>

namespace xf {

namespace {

// Energy spectrum shape, src/Fenergy.cpp:16-23.  The normaliser 18.9686 is the
// reference's hard-coded F2(eta=3); it cancels after the discrete
// normalisation of fv.
double fq(double q, double T, double eta)
{
    return (1. / 18.9686) * (1. / (T * T * T)) * ((q * q) / (std::exp(q / T - eta) + 1.));
}

// Mean energy on an 800-bin midpoint grid, src/Fenergy.cpp:25-41.
double avg_energy(const xf_config& c, int p)
{
    const int eb = 800;
    const double de = (c.E1 - c.E0) / eb;
    const double first = c.E0 + de * .5;
    double norm = 0., weighted = 0.;
    for (int e = 0; e < eb; ++e) {
        const double q = first + e * de;
        const double f = fq(q, c.Tv[p], c.eta[p]);
        norm += f;
        weighted += f * q;
    }
    return weighted / norm;
}

}  // namespace

void build_tables(const xf_config& c, Tables& t)
{
    const int ne = c.ebins;
    t.ne = ne;
    t.dE = (c.E1 - c.E0) / ne;  // fed::init, src/Fenergy.cpp:44-47
    for (int p = 0; p < 4; ++p) t.Ev[p] = avg_energy(c, p);
    for (int p = 0; p < 4; ++p) t.LE[p] = c.Lv[p] / t.Ev[p];

    // fv and hvac, src/NBeam.cpp:162-208: midpoint energies, spectra normalised
    // by their discrete sum, vacuum term (-cos 2theta, sin 2theta) * dm2/(4q).
    t.fv.assign(4 * (size_t)ne, 0.);
    t.hvac.assign(2 * (size_t)ne, 0.);
    double sum[4] = {0., 0., 0., 0.};
    const double first = c.E0 + t.dE * .5;
    for (int e = 0; e < ne; ++e) {
        const double q = first + e * t.dE;
        for (int p = 0; p < 4; ++p) {
            t.fv[(size_t)p * ne + e] = fq(q, c.Tv[p], c.eta[p]);
            sum[p] += t.fv[(size_t)p * ne + e];
        }
        const double delta = .5 * c.dm2 / q;
        t.hvac[2 * (size_t)e] = -std::cos(c.theta2) * delta * .5;
        t.hvac[2 * (size_t)e + 1] = std::sin(c.theta2) * delta * .5;
    }
    for (int p = 0; p < 4; ++p) sum[p] = 1. / sum[p];
    for (int p = 0; p < 4; ++p)
        for (int e = 0; e < ne; ++e) t.fv[(size_t)p * ne + e] *= sum[p];

    // Polar grid uniform in sin^2(theta_R): the reference accumulates the bin
    // centres by repeated subtraction, which is reproduced exactly here because
    // the angle tables at radius r are built from these values.  SA has one
    // trajectory and does not read them; a one-bin grid keeps the sizes
    // consistent with beam_dims().
    int A, P_;
    beam_dims(c, A, P_);
    t.cos2R.assign(A, 0.);
    t.dcos2R.assign(A, 0.);
    t.sinR.assign(A, 0.);
    const double dct = (1. - 0.) / A;
    t.cos2R[0] = 1. - dct * .5;
    t.sinR[0] = std::sqrt(1. - t.cos2R[0]);
    t.dcos2R[0] = dct;
    double ct = t.cos2R[0] - dct;
    for (int i = 1; i < A; ++i, ct -= dct) {
        t.cos2R[i] = ct;
        t.sinR[i] = std::sqrt(1. - t.cos2R[i]);
        t.dcos2R[i] = dct;
    }

    t.cosphi.clear();
    t.sinphi.clear();
    if (c.geometry == XF_GEOM_MAA) {
        // Azimuth bins over [0, 2pi) with the truncated pi (src/Phy_MAA.cpp:176-185).
        const int P = c.pbins;
        const double dphi = (kPi * 2.) / P;
        t.dphi = dphi;
        double phi = dphi * .5;
        t.cosphi.resize(P);
        t.sinphi.resize(P);
        for (int p = 0; p < P; ++p, phi += dphi) {
            t.sinphi[p] = std::sin(phi);
            t.cosphi[p] = std::cos(phi);
        }
        // src/Phy_MAA.cpp:297-298
        t.integ_coef = ((kSqrt2 * kGF) / (4. * kPi * kPi * c.Rv * c.Rv)) * dphi;
    } else {
        // src/Phy_MA.cpp:271-272; SA the same (src/Phy_SA.cpp:167-168)
        t.integ_coef = (kSqrt2 * kGF) / (2. * kPi * c.Rv * c.Rv);
    }

    // src/Matt.cpp:22-29
    t.mat_coeff = kSqrt2 * kGF * c.Ye;
    const double M = c.Mns / 1.4;
    const double s = 100. / c.S;
    t.nbfar_coeff = 4.2E+45 * c.gs * (M * M * M) * (s * s * s * s);
}

double matter_hm(const xf_config& c, const Tables& t, double r)
{
    if (!c.has_matter) return 0.;
    const double R = 10. / r;
    const double far = t.nbfar_coeff * (R * R * R);
    const double near = c.nb0 * std::exp((c.Rv - r) / c.hNS);
    return t.mat_coeff * (far + near) * .5;
}

namespace {
uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ULL;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
}  // namespace

double noise_u01(uint64_t seed, uint64_t beam, uint64_t e, uint64_t k)
{
    const uint64_t h = splitmix64(seed ^ splitmix64((beam << 24) ^ (e << 1) ^ k));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

void initial_state(int nbeams, int ne, uint64_t seed, double amp, std::vector<double>& psi)
{
    psi.assign((size_t)nbeams * 4 * ne, 0.);
    for (int b = 0; b < nbeams; ++b) {
        const int p = b % 4;
        double* ar = &psi[((size_t)b * 4 + 0) * ne];
        double* ai = &psi[((size_t)b * 4 + 1) * ne];
        double* br = &psi[((size_t)b * 4 + 2) * ne];
        double* bi = &psi[((size_t)b * 4 + 3) * ne];
        for (int e = 0; e < ne; ++e) {
            double eps = 0., eta = 0.;
            if (amp != 0.) {
                eps = (noise_u01(seed, b, e, 0) - 0.5) * amp;
                eta = (noise_u01(seed, b, e, 1) - 0.5) * amp;
            }
            const double one_sq = std::sqrt(1. - eps * eps - eta * eta);
            ar[e] = (p < 2) ? one_sq : eps;
            ai[e] = 0.;
            br[e] = (p < 2) ? eps : one_sq;
            bi[e] = eta;
        }
    }
}

}  // namespace xf

// ------------------------------------------------------------------ C ABI (host-only)

extern "C" int xf_host_tables(const xf_config* c, double* fv, double* hvac, double* LE, double* Ev)
{
    if (!c || c->ebins <= 0 || (c->geometry != XF_GEOM_SA && c->abins <= 0)) return XF_EINVAL;
    xf::Tables t;
    xf::build_tables(*c, t);
    if (fv) std::copy(t.fv.begin(), t.fv.end(), fv);
    if (hvac) std::copy(t.hvac.begin(), t.hvac.end(), hvac);
    if (LE) std::copy(t.LE, t.LE + 4, LE);
    if (Ev) std::copy(t.Ev, t.Ev + 4, Ev);
    return XF_OK;
}

extern "C" int xf_host_matter(const xf_config* c, double r, double* hm)
{
    if (!c || !hm || c->ebins <= 0 || (c->geometry != XF_GEOM_SA && c->abins <= 0)) return XF_EINVAL;
    xf::Tables t;
    xf::build_tables(*c, t);
    *hm = xf::matter_hm(*c, t, r);
    return XF_OK;
}

extern "C" int xf_host_initial_state(const xf_config* c, uint64_t seed, double amp, double* psi)
{
    if (!c || !psi || c->ebins <= 0 || (c->geometry != XF_GEOM_SA && c->abins <= 0)) return XF_EINVAL;
    int A, P;
    xf::beam_dims(*c, A, P);
    std::vector<double> v;
    xf::initial_state(A * P * 4, c->ebins, seed, amp, v);
    std::copy(v.begin(), v.end(), psi);
    return XF_OK;
}
