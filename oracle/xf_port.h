/*
 * Oracle (test infrastructure only; never linked into the product).
 *
 * Plain-C restatement of the reference's per-radius-step hot path for the
 * bulb-model MA, MAA and single-angle SA geometries, used as the checker for the CUDA path and
 * as the timed CPU baseline where the reference itself cannot be compiled.
 * Every function cites the reference file:line it restates.  The restatement is
 * pinned against outputs of the reference itself (oracle/_ref, built from the
 * reference's own sources by oracle/Makefile) through the fixtures in
 * tests/golden/.
 */
#ifndef XF_PORT_H_
#define XF_PORT_H_
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xfp_sim xfp_sim;

/* Parse a reference-format config file (src/Parser.cpp:25-127) and build the
 * module state (nbm::init, phy::init, nmr::init, matt::init:
 * src/NBGroup.cpp:129-139).  Returns NULL on failure. */
xfp_sim* xfp_create(const char* config_path);
void xfp_destroy(xfp_sim* s);

int xfp_geometry(const xfp_sim* s);   /* 0 = MA, 1 = MAA, 2 = SA */
int xfp_nbeams(const xfp_sim* s);     /* theta * phi * 4 */
int xfp_ebins(const xfp_sim* s);
int xfp_abins(const xfp_sim* s);
int xfp_pbins(const xfp_sim* s);
/* r0, rn, dr0, eps0, ksi, max_dr, Ts, Tn, seed, noise_amp */
void xfp_params(const xfp_sim* s, double out[10]);

/* Tables: fv[4][ne], hvac[2*ne], LE[4], Ev[4]. */
void xfp_tables(const xfp_sim* s, double* fv, double* hvac, double* LE, double* Ev);
/* Matter term hm(r) = matt::getHm (src/Matt.cpp:58-64). */
double xfp_hm(const xfp_sim* s, double r);

/* State IO in the NetCDF psi layout [beam][comp][ebin]; which = 0,1,3,4. */
void xfp_set_state(xfp_sim* s, const double* psi);
void xfp_get_state(const xfp_sim* s, int which, double* psi);
/* Per-beam cached energy sums hSumMat (4 doubles per beam) of buffer which. */
void xfp_get_esum(const xfp_sim* s, int which, double* out);
/* Seeded initial noise (counter-based splitmix64 generator). */
void xfp_noise(xfp_sim* s, uint64_t seed, double amp);

/* Angle tables and Hamiltonian on buffer `which` at stage point pt, after
 * calcAngleBins(r,0..2) and calcDeltaLs (src/Nmr.cpp:167-173).
 * cos/sin/dcos/dl: [3][abins]; hvv: [abins*pbins][4]. */
void xfp_probe(xfp_sim* s, double r, double dr, double* cosb, double* sinb, double* dcosb, double* dl);
void xfp_calc_hvv(xfp_sim* s, int which, int pt, double* hvv);

/* One stepper iteration at (r, dr): stages S1..S11 and the error sweep
 * (src/Nmr.cpp:153-206).  Returns Max_err; psi0 is untouched. */
double xfp_iterate(xfp_sim* s, double r, double dr);
/* Accept: swap psi0 and psi4 (src/Nmr.cpp:227-233). */
void xfp_accept(xfp_sim* s);

/* Full evolution loop (src/Nmr.cpp:89-262) from (r0, dr0) with the config's
 * Rn/Ts (max_iters < 0 -> config Ts).  Writes up to log_cap accepted records
 * (itr, r_after, dr_used) into log.  Returns total iterations; *n_acc,
 * *r_end, *dr_end receive accepted count and the final r and dr. */
long xfp_run(xfp_sim* s, double r0, double dr0, long max_iters, double* log, long log_cap,
             long* n_acc, double* r_end, double* dr_end);

/* Replay: apply the given accepted (r_before, dr) pairs as forced steps. */
void xfp_replay(xfp_sim* s, const double* r_before, const double* dr, long n);

#ifdef __cplusplus
}
#endif
#endif
