// Host-side physics set-up shared by every GPU path: unit constants, energy
// spectra and vacuum Hamiltonian tables, angle grids at the neutrinosphere,
// Hamiltonian coefficients, the matter profile and the seeded initial noise.
// All of it runs once per run (or per radius for the matter term) on the host,
// as in the reference, and is uploaded to the device as read-only tables.
#pragma once
#include <cstdint>
#include <vector>

#include "xflat_gpu.h"

namespace xf {

// include/global.h:43-46
constexpr double kErgS = 1.053613095584080e+16;  // erg/s -> km^-2
constexpr double kMeV = 5.067731161976211e+15;   // MeV -> km^-1
constexpr double kMeV2 = 3.893793036626876e-32;  // MeV^-2 -> km^2
constexpr double kEV2 = 2.568189913006477e+19;   // eV^2 -> km^-2
// include/Util.h:15-22.  The reference uses truncated constants; they enter the
// Hamiltonian coefficients and the azimuth grid, so they are kept verbatim.
constexpr double kSqrt2 = 1.41421356237;
constexpr double kPi = 3.14159265359;
constexpr double kGF = 1.16637E-11 * kMeV2;

// Angle bins A and azimuth bins P of a configuration: SA has one trajectory
// whatever Abins says (src/Phy_SA.cpp:150-184, beam_len = 2 Flvs), MA one
// azimuth bin, MAA Pbins.  Beams = A P 4.
inline void beam_dims(const xf_config& c, int& A, int& P)
{
    A = c.geometry == XF_GEOM_SA ? 1 : c.abins;
    P = c.geometry == XF_GEOM_MAA ? c.pbins : 1;
}

struct Tables {
    int ne = 0;
    double dE = 0;
    double Ev[4] = {0, 0, 0, 0};     // <E> per particle (src/Fenergy.cpp:25-41)
    double LE[4] = {0, 0, 0, 0};     // L/<E> (src/Phy_MA.cpp:280-282)
    std::vector<double> fv;          // [4][ne] normalised spectra (src/NBeam.cpp:162-208)
    std::vector<double> hvac;        // [ne][2] vacuum Hamiltonian (src/NBeam.cpp:179-185)
    // angle grids at the neutrinosphere (src/Phy_MA.cpp:141-164, src/Phy_MAA.cpp:144-186)
    std::vector<double> cos2R, dcos2R, sinR;  // [abins]
    std::vector<double> cosphi, sinphi;       // [pbins] (MAA), empty for MA
    double dphi = 0;
    double integ_coef = 0;   // kappa (MA) or kappa' * dphi (MAA)
    // matter profile coefficients (src/Matt.cpp:22-29)
    double mat_coeff = 0, nbfar_coeff = 0;
};

// Builds every table above from a configuration.
void build_tables(const xf_config& c, Tables& t);

// matt::getHm (src/Matt.cpp:31-64): 0.5 * sqrt2 GF Ye (nb_far + nb_near).
double matter_hm(const xf_config& c, const Tables& t, double r);

// Counter-based uniform in [0,1): splitmix64 keyed on (seed, beam, ebin, k).
double noise_u01(uint64_t seed, uint64_t beam, uint64_t e, uint64_t k);

// Initial beam state in the psi layout [beam][comp][ebin]: pure flavor states
// (src/NBeam.cpp:246-276) with optional seeded noise of amplitude amp.
void initial_state(int nbeams, int ne, uint64_t seed, double amp, std::vector<double>& psi);

}  // namespace xf
