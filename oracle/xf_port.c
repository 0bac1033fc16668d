/*
 * Oracle (test infrastructure only; never linked into the product).
 *
 * Plain-C restatement of the reference's hot path (bulb-model MA/MAA and single-angle SA geometry,
 * the NBeam per-bin SU(2) kernels and the adaptive three-point stepper).  The
 * loop structure (OpenMP over angle bins, omp simd over energy bins) and the
 * floating-point operation order follow the reference line by line, so the
 * results agree with the compiled reference to rounding; tests/golden/ pins it
 * against outputs of the reference itself.
 */
#define _POSIX_C_SOURCE 200809L
#include "xf_port.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* include/global.h:43-46 */
#define ERG_S 1.053613095584080e+16
#define MEV 5.067731161976211e+15
#define MEV_2 3.893793036626876e-32
#define EV2 2.568189913006477e+19
/* include/Util.h:15-22 (truncated constants, kept for parity) */
#define U_SQRT2 1.41421356237
#define U_PI 3.14159265359
#define U_GF (1.16637E-11 * MEV_2)

struct xfp_sim {
    int geom;
    /* configuration (src/Parser.cpp:40-123; units converted at parse time) */
    double eps0, ksi, mu, R0, Rn, dr0, maxdr, E0, E1, Ye, Rv, Mns, gs, S, hNS, nb0;
    double theta, theta2, dm2;
    int Ts, Tn, hasMatter, Abins, Pbins, Ebins, Flvs;
    double Lv[4], Tv[4], eta[4];
    uint64_t seed;
    double noise_amp;
    /* nbm / fed (src/NBeam.cpp:138-209, src/Fenergy.cpp) */
    double dE, Ev[4];
    double* fq[4];
    double* hvac;
    /* phy (src/Phy_MA.cpp:233-284, src/Phy_MAA.cpp:247-304) */
    int tet, pb, nbeams, ne;
    double *Cos2R, *dCos2R, *SinR, *sinphi, *cosphi, dPhi;
    double *cosb, *sinb, *dcosb, *dl; /* [3][tet] */
    double rpt[3];                     /* SA: radius of each stage point (src/Phy_SA.cpp:121-124) */
    double integ_coef, LE[4];
    /* matt (src/Matt.cpp:22-29) */
    double mat_coeff, nbfar_coeff;
    /* beam buffers psi[k] = [beam][comp][ebin], k in {0,1,3,4}; hsum = hSumMat */
    double* psi[5];
    double* hsum[5];
    int i0, i4; /* current roles of the psi0 / psi4 buffers (pointer swap) */
};

static void* xalloc(size_t n)
{
    void* p = NULL;
    if (posix_memalign(&p, 64, n ? n : 64) != 0) return NULL;
    memset(p, 0, n ? n : 64);
    return p;
}

/* ------------------------------------------------------------------ parser */

static void set_key(xfp_sim* s, const char* k, const char* v)
{
    double d = strtod(v, NULL);
    long i = strtol(v, NULL, 10);
    /* src/Parser.cpp:62-123 */
    if (!strcmp(k, "hasMatter=")) s->hasMatter = (int)i;
    else if (!strcmp(k, "eps0=")) s->eps0 = d;
    else if (!strcmp(k, "ksi=")) s->ksi = d;
    else if (!strcmp(k, "mu=")) s->mu = d;
    else if (!strcmp(k, "Tn=")) s->Tn = (int)i;
    else if (!strcmp(k, "Ts=")) s->Ts = (int)i;
    else if (!strcmp(k, "R0=")) s->R0 = d;
    else if (!strcmp(k, "Rn=")) s->Rn = d;
    else if (!strcmp(k, "dr=")) s->dr0 = d;
    else if (!strcmp(k, "max_dr=")) s->maxdr = d;
    else if (!strcmp(k, "E0=")) s->E0 = d * MEV;
    else if (!strcmp(k, "E1=")) s->E1 = d * MEV;
    else if (!strcmp(k, "Pbins=")) s->Pbins = (int)i;
    else if (!strcmp(k, "Abins=")) s->Abins = (int)i;
    else if (!strcmp(k, "Ebins=")) s->Ebins = (int)i;
    else if (!strcmp(k, "Flvs=")) s->Flvs = (int)i;
    else if (!strcmp(k, "Ye=")) s->Ye = d;
    else if (!strcmp(k, "Rv=")) s->Rv = d;
    else if (!strcmp(k, "Mns=")) s->Mns = d;
    else if (!strcmp(k, "gs=")) s->gs = d;
    else if (!strcmp(k, "S=")) s->S = d;
    else if (!strcmp(k, "hNS=")) s->hNS = d;
    else if (!strcmp(k, "nb0=")) s->nb0 = d * 1.E+15;
    else if (!strcmp(k, "theta=")) { s->theta = d; s->theta2 = d * 2; }
    else if (!strcmp(k, "dm2=")) s->dm2 = d * EV2;
    else if (!strcmp(k, "Lve=")) s->Lv[0] = d * ERG_S;
    else if (!strcmp(k, "Lv_e=")) s->Lv[1] = d * ERG_S;
    else if (!strcmp(k, "Lvt=")) s->Lv[2] = d * ERG_S;
    else if (!strcmp(k, "Lv_t=")) s->Lv[3] = d * ERG_S;
    else if (!strcmp(k, "Tve=")) s->Tv[0] = d * MEV;
    else if (!strcmp(k, "Tv_e=")) s->Tv[1] = d * MEV;
    else if (!strcmp(k, "Tvt=")) s->Tv[2] = d * MEV;
    else if (!strcmp(k, "Tv_t=")) s->Tv[3] = d * MEV;
    else if (!strcmp(k, "eta_ve=")) s->eta[0] = d;
    else if (!strcmp(k, "eta_v_e=")) s->eta[1] = d;
    else if (!strcmp(k, "eta_vt=")) s->eta[2] = d;
    else if (!strcmp(k, "eta_v_t=")) s->eta[3] = d;
    /* extension keys (skipped by the reference parser) */
    else if (!strcmp(k, "geometry=")) {
        if ((v[0] == 'M' || v[0] == 'm') && (v[1] == 'A' || v[1] == 'a') && (v[2] == 'A' || v[2] == 'a')) s->geom = 1;
        else if ((v[0] == 'S' || v[0] == 's') && (v[1] == 'A' || v[1] == 'a')) s->geom = 2;
        else s->geom = 0;
    }
    else if (!strcmp(k, "seed=")) s->seed = strtoull(v, NULL, 10);
    else if (!strcmp(k, "noise_amp=")) s->noise_amp = d;
}

static int parse_file(xfp_sim* s, const char* path)
{
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    char line[1024];
    while (fgets(line, sizeof line, f)) {
        char key[256], val[256];
        val[0] = 0;
        int n = sscanf(line, "%255s %255s", key, val);
        if (n < 1 || key[0] == '#') continue;
        set_key(s, key, val);
    }
    fclose(f);
    return 0;
}

/* ------------------------------------------------------------ energy/nbm */

/* src/Fenergy.cpp:16-23 */
static double fq(double q, double Tv, double eta_v)
{
    return (1. / 18.9686) * (1. / (Tv * Tv * Tv)) * ((q * q) / (exp(q / Tv - eta_v) + 1.));
}

/* src/Fenergy.cpp:25-41 */
static double avg_energy(const xfp_sim* s, int p)
{
    const int Eb = 800;
    double de = (s->E1 - s->E0) / Eb;
    double frst = s->E0 + de * .5;
    double avg = 0., Eavg = 0.;
    for (int e = 0; e < Eb; ++e) {
        double q = frst + e * de;
        double fe = fq(q, s->Tv[p], s->eta[p]);
        avg += fe;
        Eavg += fe * q;
    }
    return Eavg / avg;
}

/* src/NBeam.cpp:138-209 */
static void nbm_init(xfp_sim* s)
{
    const int ne = s->ne;
    s->dE = (s->E1 - s->E0) / ne;
    for (int p = 0; p < 4; ++p) s->Ev[p] = avg_energy(s, p);
    for (int p = 0; p < 4; ++p) s->fq[p] = (double*)xalloc(ne * sizeof(double));
    s->hvac = (double*)xalloc(2 * ne * sizeof(double));
    double sum[4] = {0., 0., 0., 0.};
    double frst = s->E0 + s->dE * .5;
    for (int e = 0; e < ne; ++e) {
        double q = frst + e * s->dE;
        for (int p = 0; p < 4; ++p) {
            s->fq[p][e] = fq(q, s->Tv[p], s->eta[p]);
            sum[p] += s->fq[p][e];
        }
        double delta = .5 * s->dm2 / q;
        double th = s->theta2;
        s->hvac[2 * e] = -cos(th) * delta * .5;
        s->hvac[2 * e + 1] = sin(th) * delta * .5;
    }
    for (int p = 0; p < 4; ++p) sum[p] = 1. / sum[p];
    for (int e = 0; e < ne; ++e)
        for (int p = 0; p < 4; ++p) s->fq[p][e] *= sum[p];
}

/* ------------------------------------------------------------ matter */

/* src/Matt.cpp:22-29 */
static void matt_init(xfp_sim* s)
{
    s->mat_coeff = U_SQRT2 * U_GF * s->Ye;
    double M = s->Mns / 1.4;
    double sr = 100. / s->S;
    s->nbfar_coeff = 4.2E+45 * s->gs * (M * M * M) * (sr * sr * sr * sr);
}

/* src/Matt.cpp:31-64 */
double xfp_hm(const xfp_sim* s, double r)
{
    if (!s->hasMatter) return 0.;
    double R = 10. / r;
    double far = s->nbfar_coeff * (R * R * R);
    double near = s->nb0 * exp((s->Rv - r) / s->hNS);
    return s->mat_coeff * (far + near) * .5;
}

/* ------------------------------------------------------------ geometry */

/* src/Phy_MA.cpp:141-164 and src/Phy_MAA.cpp:144-186 */
static void init_angles(xfp_sim* s)
{
    const int A = s->Abins;
    s->Cos2R = (double*)xalloc(A * sizeof(double));
    s->dCos2R = (double*)xalloc(A * sizeof(double));
    s->SinR = (double*)xalloc(A * sizeof(double));
    double dct = (1. - 0.) / A;
    s->Cos2R[0] = 1. - dct * .5;
    s->SinR[0] = sqrt(1. - s->Cos2R[0]);
    s->dCos2R[0] = dct;
    double ct = s->Cos2R[0] - dct;
    for (int i = 1; i < A; ++i, ct -= dct) {
        s->Cos2R[i] = ct;
        s->SinR[i] = sqrt(1. - s->Cos2R[i]);
        s->dCos2R[i] = dct;
    }
    const int P = s->pb;
    s->sinphi = (double*)xalloc(P * sizeof(double));
    s->cosphi = (double*)xalloc(P * sizeof(double));
    if (s->geom == 1) {
        double dphi = (U_PI * 2.) / P;
        s->dPhi = dphi;
        double phi = dphi * .5;
        for (int p = 0; p < P; ++p, phi += dphi) {
            s->sinphi[p] = sin(phi);
            s->cosphi[p] = cos(phi);
        }
    }
}

/* SA dilution factor D(r) = (1 - sqrt(1 - (Rv/r)^2))^2 / 2, src/Phy_SA.cpp:250-256 */
static double sa_D(double Rv, double r)
{
    double R = Rv / r;
    double tm = 1. - sqrt(1. - (R * R));
    return 0.5 * (tm * tm);
}

/* src/Phy_MA.cpp:172-196, src/Phy_MAA.cpp:194-210; SA keeps only the radius
 * (src/Phy_SA.cpp:121-124).  For SA the tables report cos = sin = 0 and the
 * dilution factor D(r) in the weight slot, the form in which an MA-shaped
 * moment H = kappa (J0 - cos J1) with J0 = sum w N reduces to SA's
 * kappa D(r) sum N. */
static void calc_angle_bins(xfp_sim* s, double r, int step)
{
    const int T = s->tet;
    if (s->geom == 2) {
        s->rpt[step] = r;
        s->cosb[step] = 0.;
        s->sinb[step] = 0.;
        s->dcosb[step] = sa_D(s->Rv, r);
        return;
    }
    double ra = s->Rv / r;
    double r2 = ra * ra;
#pragma omp parallel for
    for (int ang = 0; ang < T; ++ang) {
        int idx = step * T + ang;
        s->cosb[idx] = sqrt(1. - r2 * (1. - s->Cos2R[ang]));
        s->sinb[idx] = ra * s->SinR[ang];
        s->dcosb[idx] = .5 * (1. / s->cosb[idx]) * r2 * s->dCos2R[ang];
    }
}

/* src/Phy_MA.cpp:218-227 (start-point cos), src/Phy_MAA.cpp:232-241 (mean cos) */
static void calc_delta_ls(xfp_sim* s, double dr, int cur, int sp, int ep)
{
    const int T = s->tet;
    if (s->geom == 2) { /* src/Phy_SA.cpp:144-147 */
        s->dl[cur] = dr;
        return;
    }
#pragma omp parallel for
    for (int ang = 0; ang < T; ++ang) {
        if (s->geom == 1)
            s->dl[cur * T + ang] = dr / ((s->cosb[sp * T + ang] + s->cosb[ep * T + ang]) * .5);
        else
            s->dl[cur * T + ang] = dr / (s->cosb[sp * T + ang]);
    }
}

/* ------------------------------------------------------------ beam kernel */

/* src/NBeam.cpp:360-393 */
static inline void beam_U(double dr, double h_r0, double h_r1, double h_i1, double a_r, double a_i,
                          double b_r, double b_i, double* n_ar, double* n_ai, double* n_br, double* n_bi)
{
    double lambda = sqrt(h_r0 * h_r0 + (h_r1 * h_r1 + h_i1 * h_i1));
    double ldr = lambda * dr;
    double cosCoef = cos(ldr);
    double sinCoef = sin(ldr) / lambda;
    double mat0 = cosCoef;
    double mat1 = -h_r0 * sinCoef;
    double mat2 = h_i1 * sinCoef;
    double mat3 = -h_r1 * sinCoef;
    double mat4 = -mat2;
    double mat5 = mat3;
    double mat6 = mat0;
    double mat7 = -mat1;
    double r00r = mat0 * a_r - mat1 * a_i, r00i = mat0 * a_i + mat1 * a_r;
    double r01r = mat2 * b_r - mat3 * b_i, r01i = mat2 * b_i + mat3 * b_r;
    double r10r = mat4 * a_r - mat5 * a_i, r10i = mat4 * a_i + mat5 * a_r;
    double r11r = mat6 * b_r - mat7 * b_i, r11i = mat6 * b_i + mat7 * b_r;
    *n_ar = r00r + r01r;
    *n_ai = r00i + r01i;
    *n_br = r10r + r11r;
    *n_bi = r10i + r11i;
}

/* particle-dependent Hamiltonian offsets, src/NBeam.cpp:602-607 */
static inline void hm_vv(int p, const double* hvv, double hmatt, double hmvv[4])
{
    hmvv[0] = (p % 2) ? -(hvv[0] + hmatt) : (hvv[0] + hmatt);
    hmvv[1] = hvv[1];
    hmvv[2] = (p % 2) ? -hvv[2] : hvv[2];
    hmvv[3] = hvv[3];
}

#define BEAM(buf, b, c) ((buf) + ((size_t)(b) * 4 + (c)) * ne)

/* src/NBeam.cpp:588-646: out = U(in); hsum(out) */
static void evolve_bins_hvv(const xfp_sim* s, double* out, double* hs, const double* in, int p, double dr,
                            const double* hvv, double hmatt, int b)
{
    const int ne = s->ne;
    double* ar = BEAM(out, b, 0); double* ai = BEAM(out, b, 1);
    double* br = BEAM(out, b, 2); double* bi = BEAM(out, b, 3);
    const double* iar = BEAM(in, b, 0); const double* iai = BEAM(in, b, 1);
    const double* ibr = BEAM(in, b, 2); const double* ibi = BEAM(in, b, 3);
    const double* fv = s->fq[p];
    const double* hv = s->hvac;
    double hmvv[4];
    hm_vv(p, hvv, hmatt, hmvv);
    double r0 = 0., r1 = 0., r2 = 0., r3 = 0.;
#pragma omp simd reduction(+ : r0, r1, r2, r3)
    for (int e = 0; e < ne; ++e) {
        double h0 = hv[2 * e] + hmvv[0];
        double h2 = hv[2 * e + 1] + hmvv[2];
        double nar, nai, nbr, nbi;
        beam_U(dr, h0, h2, hmvv[3], iar[e], iai[e], ibr[e], ibi[e], &nar, &nai, &nbr, &nbi);
        ar[e] = nar; ai[e] = nai; br[e] = nbr; bi[e] = nbi;
        double d0 = .5 * ((nar * nar + nai * nai) - (nbr * nbr + nbi * nbi));
        double d2 = nar * nbr - nai * (-nbi);
        double d3 = nar * (-nbi) + nai * nbr;
        r0 += d0 * fv[e];
        r1 += 0. * fv[e];
        r2 += d2 * fv[e];
        r3 += d3 * fv[e];
    }
    hs[4 * b + 0] = r0; hs[4 * b + 1] = r1; hs[4 * b + 2] = r2; hs[4 * b + 3] = r3;
}

/* src/NBeam.cpp:462-514: out = U(in); avg = (out + avg)/2 */
static void evolve_bins_avg(const xfp_sim* s, double* out, const double* in, double* avg, int p, double dr,
                            const double* hvv, double hmatt, int b)
{
    const int ne = s->ne;
    double* ar = BEAM(out, b, 0); double* ai = BEAM(out, b, 1);
    double* br = BEAM(out, b, 2); double* bi = BEAM(out, b, 3);
    const double* iar = BEAM(in, b, 0); const double* iai = BEAM(in, b, 1);
    const double* ibr = BEAM(in, b, 2); const double* ibi = BEAM(in, b, 3);
    double* var = BEAM(avg, b, 0); double* vai = BEAM(avg, b, 1);
    double* vbr = BEAM(avg, b, 2); double* vbi = BEAM(avg, b, 3);
    const double* hv = s->hvac;
    double hmvv[4];
    hm_vv(p, hvv, hmatt, hmvv);
#pragma omp simd
    for (int e = 0; e < ne; ++e) {
        double h0 = hv[2 * e] + hmvv[0];
        double h2 = hv[2 * e + 1] + hmvv[2];
        double nar, nai, nbr, nbi;
        beam_U(dr, h0, h2, hmvv[3], iar[e], iai[e], ibr[e], ibi[e], &nar, &nai, &nbr, &nbi);
        ar[e] = nar; ai[e] = nai; br[e] = nbr; bi[e] = nbi;
        var[e] = (nar + var[e]) * .5;
        vai[e] = (nai + vai[e]) * .5;
        vbr[e] = (nbr + vbr[e]) * .5;
        vbi[e] = (nbi + vbi[e]) * .5;
    }
}

/* src/NBeam.cpp:690-736: io = U(io); avg = (io + avg)/2 */
static void evolve_bins_avg_inplace(const xfp_sim* s, double* io, double* avg, int p, double dr,
                                    const double* hvv, double hmatt, int b)
{
    evolve_bins_avg(s, io, io, avg, p, dr, hvv, hmatt, b);
}

/* src/NBeam.cpp:812-840 */
static void calc_esum(const xfp_sim* s, const double* buf, double* hs, int b)
{
    const int ne = s->ne;
    const double* ar = BEAM(buf, b, 0); const double* ai = BEAM(buf, b, 1);
    const double* br = BEAM(buf, b, 2); const double* bi = BEAM(buf, b, 3);
    const double* fv = s->fq[b % 4];
    double r0 = 0., r1 = 0., r2 = 0., r3 = 0.;
#pragma omp simd reduction(+ : r0, r1, r2, r3)
    for (int e = 0; e < ne; ++e) {
        double d0 = .5 * ((ar[e] * ar[e] + ai[e] * ai[e]) - (br[e] * br[e] + bi[e] * bi[e]));
        double d2 = ar[e] * br[e] - ai[e] * (-bi[e]);
        double d3 = ar[e] * (-bi[e]) + ai[e] * br[e];
        r0 += d0 * fv[e];
        r1 += 0. * fv[e];
        r2 += d2 * fv[e];
        r3 += d3 * fv[e];
    }
    hs[4 * b + 0] = r0; hs[4 * b + 1] = r1; hs[4 * b + 2] = r2; hs[4 * b + 3] = r3;
}

/* src/NBeam.cpp:903-938: err of buf (this) against ref (beam), plus hsum(buf) */
static double calc_err_hvv(const xfp_sim* s, const double* buf, const double* ref, double* hs, int b)
{
    const int ne = s->ne;
    const double* ar = BEAM(buf, b, 0); const double* ai = BEAM(buf, b, 1);
    const double* br = BEAM(buf, b, 2); const double* bi = BEAM(buf, b, 3);
    const double* mar = BEAM(ref, b, 0); const double* mai = BEAM(ref, b, 1);
    const double* mbr = BEAM(ref, b, 2); const double* mbi = BEAM(ref, b, 3);
    const double* fv = s->fq[b % 4];
    double eps = 0., r0 = 0., r1 = 0., r2 = 0., r3 = 0.;
#pragma omp simd reduction(+ : eps, r0, r1, r2, r3)
    for (int e = 0; e < ne; ++e) {
        double x0 = ar[e] - mar[e], x1 = ai[e] - mai[e], x2 = br[e] - mbr[e], x3 = bi[e] - mbi[e];
        eps += ((x0 * x0 + x1 * x1) + (x2 * x2 + x3 * x3)) * (fv[e]);
        double d0 = .5 * ((ar[e] * ar[e] + ai[e] * ai[e]) - (br[e] * br[e] + bi[e] * bi[e]));
        double d2 = ar[e] * br[e] - ai[e] * (-bi[e]);
        double d3 = ar[e] * (-bi[e]) + ai[e] * br[e];
        r0 += d0 * fv[e];
        r1 += 0. * fv[e];
        r2 += d2 * fv[e];
        r3 += d3 * fv[e];
    }
    hs[4 * b + 0] = r0; hs[4 * b + 1] = r1; hs[4 * b + 2] = r2; hs[4 * b + 3] = r3;
    return eps;
}

/* ------------------------------------------------------------ Hamiltonian */

/* include/NBeam.h:47-53 */
static inline void upd_nu_coef(const double* nu, const double* anu, double n_cf, double an_cf, double* ret)
{
    ret[0] += nu[0] * n_cf - anu[0] * an_cf;
    ret[1] += nu[1] * n_cf - anu[1] * an_cf;
    ret[2] += nu[2] * n_cf - anu[2] * an_cf;
    ret[3] += nu[3] * n_cf + anu[3] * an_cf;
}

/* MA: src/Phy_MA.cpp:388-474 */
static void calc_hvv_ma(xfp_sim* s, const double* hs, int step, double* hvv)
{
    const int T = s->tet, F = s->Flvs;
    const double* Cos = &s->cosb[step * T];
    const double* dCos = &s->dcosb[step * T];
    double* np = (double*)xalloc((size_t)T * 4 * sizeof(double));
    double* npc = (double*)xalloc((size_t)T * 4 * sizeof(double));
#pragma omp parallel for
    for (int ang = 0; ang < T; ++ang) {
        for (int n = 0; n < F; ++n) {
            int neu = n << 1, aneu = neu + 1;
            upd_nu_coef(&hs[4 * (ang * 2 * F + neu)], &hs[4 * (ang * 2 * F + aneu)], s->LE[neu], s->LE[aneu],
                        &np[ang * 4]);
        }
        for (int z = 0; z < 4; ++z) {
            np[ang * 4 + z] *= dCos[ang];
            npc[ang * 4 + z] = np[ang * 4 + z] * Cos[ang];
        }
    }
    double part[4] = {0., 0., 0., 0.}, partc[4] = {0., 0., 0., 0.};
    for (int a = 0; a < T; ++a)
        for (int z = 0; z < 4; ++z) {
            part[z] += np[a * 4 + z];
            partc[z] += npc[a * 4 + z];
        }
    free(np);
    free(npc);
#pragma omp parallel for
    for (int ang = 0; ang < T; ++ang)
        for (int z = 0; z < 4; ++z) hvv[ang * 4 + z] = (part[z] - (partc[z] * Cos[ang])) * s->integ_coef;
}

/* MAA: src/Phy_MAA.cpp:468-621 */
static void calc_hvv_maa(xfp_sim* s, const double* hs, int step, double* hvv)
{
    const int T = s->tet, P = s->pb, F = s->Flvs, np_ = 2 * F;
    double* pt = (double*)xalloc((size_t)T * 4 * sizeof(double));
    double* cs = (double*)xalloc((size_t)T * 4 * sizeof(double));
    double* sn = (double*)xalloc((size_t)T * 4 * sizeof(double));
    double* ct = (double*)xalloc((size_t)T * 4 * sizeof(double));
#pragma omp parallel for
    for (int ang = 0; ang < T; ++ang) {
        double cosP[4] = {0., 0., 0., 0.}, sinP[4] = {0., 0., 0., 0.};
        for (int phi = 0; phi < P; ++phi) {
            double pe[4] = {0., 0., 0., 0.};
            for (int n = 0; n < F; ++n) {
                int neu = n << 1, aneu = neu + 1;
                int base = (ang * P + phi) * np_;
                upd_nu_coef(&hs[4 * (base + neu)], &hs[4 * (base + aneu)], s->LE[neu], s->LE[aneu], pe);
            }
            for (int z = 0; z < 4; ++z) {
                pt[ang * 4 + z] += pe[z];
                cosP[z] += pe[z] * s->cosphi[phi];
                sinP[z] += pe[z] * s->sinphi[phi];
            }
        }
        for (int z = 0; z < 4; ++z) {
            int idx = ang * 4 + z, aid = step * T + ang;
            pt[idx] *= s->dcosb[aid];
            cs[idx] = cosP[z] * s->sinb[aid] * s->dcosb[aid];
            sn[idx] = sinP[z] * s->sinb[aid] * s->dcosb[aid];
            ct[idx] = pt[idx] * s->cosb[aid];
        }
    }
    double J0[4], Jx[4], Jy[4], Jz[4];
    for (int z = 0; z < 4; ++z) {
        for (int ang = 1; ang < T; ++ang) {
            int idx = ang * 4 + z;
            pt[z] += pt[idx];
            cs[z] += cs[idx];
            sn[z] += sn[idx];
            ct[z] += ct[idx];
        }
        J0[z] = pt[z]; Jx[z] = cs[z]; Jy[z] = sn[z]; Jz[z] = ct[z];
    }
    free(pt); free(cs); free(sn); free(ct);
#pragma omp parallel for
    for (int ang = 0; ang < T; ++ang)
        for (int phi = 0; phi < P; ++phi) {
            int aid = step * T + ang;
            double st = s->sinb[aid], c_t = s->cosb[aid], sp = s->sinphi[phi], cp = s->cosphi[phi];
            for (int z = 0; z < 4; ++z)
                hvv[(ang * P + phi) * 4 + z] = (J0[z] - (st * cp * Jx[z] + st * sp * Jy[z] + c_t * Jz[z])) * s->integ_coef;
        }
}

/* SA: src/Phy_SA.cpp:259-281 */
static void calc_hvv_sa(xfp_sim* s, const double* hs, int step, double* hvv)
{
    for (int z = 0; z < 4; ++z) hvv[z] = 0.;
    for (int n = 0; n < s->Flvs; ++n) {
        int neu = n << 1, aneu = neu + 1;
        upd_nu_coef(&hs[4 * neu], &hs[4 * aneu], s->LE[neu], s->LE[aneu], hvv);
    }
    double coeff = s->integ_coef * sa_D(s->Rv, s->rpt[step]);
    for (int z = 0; z < 4; ++z) hvv[z] *= coeff;
}

static void calc_hvv(xfp_sim* s, const double* hs, int step, double* hvv)
{
    if (s->geom == 2) calc_hvv_sa(s, hs, step, hvv);
    else if (s->geom == 1) calc_hvv_maa(s, hs, step, hvv);
    else calc_hvv_ma(s, hs, step, hvv);
}

/* ------------------------------------------------------------ sweeps */

/* Sweep kinds mirror phy::evolveHvv and both phy::evolveAvg overloads
 * (src/Phy_MA.cpp:494-540, src/Phy_MAA.cpp:738-803). */
enum { SW_HVV, SW_AVG, SW_AVG_INPLACE };

static void sweep(xfp_sim* s, int kind, int pnt, const double* hvv, double hmatt, const double* in, double* out,
                  double* out_hs, double* avg)
{
    const int T = s->tet, P = s->pb, NP = 2 * s->Flvs;
#pragma omp parallel for
    for (int ang = 0; ang < T; ++ang) {
        double dlv = s->dl[pnt * T + ang];
        for (int phi = 0; phi < P; ++phi) {
            int aid = (ang * P + phi) * 4;
            for (int prc = 0; prc < NP; ++prc) {
                int idx = (ang * P + phi) * NP + prc;
                if (kind == SW_HVV) evolve_bins_hvv(s, out, out_hs, in, prc, dlv, &hvv[aid], hmatt, idx);
                else if (kind == SW_AVG) evolve_bins_avg(s, out, in, avg, prc, dlv, &hvv[aid], hmatt, idx);
                else evolve_bins_avg_inplace(s, out, avg, prc, dlv, &hvv[aid], hmatt, idx);
            }
        }
    }
}

/* ------------------------------------------------------------ public API */

xfp_sim* xfp_create(const char* path)
{
    xfp_sim* s = (xfp_sim*)calloc(1, sizeof(xfp_sim));
    if (!s) return NULL;
    s->Flvs = 2;
    s->Pbins = 1;
    if (parse_file(s, path) != 0 || s->Abins <= 0 || s->Ebins <= 0 || s->Flvs != 2) {
        free(s);
        return NULL;
    }
    if (s->geom == 0) s->Pbins = s->Pbins > 0 ? s->Pbins : 1;
    /* SA: one beam per particle whatever Abins says (src/Phy_SA.cpp:150-184) */
    s->tet = (s->geom == 2) ? 1 : s->Abins;
    s->pb = (s->geom == 1) ? s->Pbins : 1;
    s->ne = s->Ebins;
    s->nbeams = s->tet * s->pb * 2 * s->Flvs;
    nbm_init(s);
    init_angles(s);
    if (s->geom == 1)
        s->integ_coef = ((U_SQRT2 * U_GF) / (4. * U_PI * U_PI * s->Rv * s->Rv)) * s->dPhi;
    else
        s->integ_coef = (U_SQRT2 * U_GF) / (2. * U_PI * s->Rv * s->Rv); /* MA :271, SA src/Phy_SA.cpp:167-168 */
    for (int i = 0; i < 4; ++i) s->LE[i] = s->Lv[i] / s->Ev[i];
    matt_init(s);
    const size_t T3 = (size_t)3 * s->tet * sizeof(double);
    s->cosb = (double*)xalloc(T3);
    s->sinb = (double*)xalloc(T3);
    s->dcosb = (double*)xalloc(T3);
    s->dl = (double*)xalloc(T3);
    const size_t nb = (size_t)s->nbeams * 4 * s->ne * sizeof(double);
    const int ids[4] = {0, 1, 3, 4};
    for (int k = 0; k < 4; ++k) {
        s->psi[ids[k]] = (double*)xalloc(nb);
        s->hsum[ids[k]] = (double*)xalloc((size_t)s->nbeams * 4 * sizeof(double));
        /* NBeam constructor, src/NBeam.cpp:246-276 (PERTERB off) */
        for (int b = 0; b < s->nbeams; ++b) {
            int p = b % 4;
            const int ne = s->ne;
            for (int e = 0; e < s->ne; ++e) {
                BEAM(s->psi[ids[k]], b, 0)[e] = (p < 2) ? 1. : 0.;
                BEAM(s->psi[ids[k]], b, 2)[e] = (p < 2) ? 0. : 1.;
            }
        }
    }
    s->i0 = 0;
    s->i4 = 4;
    for (int b = 0; b < s->nbeams; ++b) calc_esum(s, s->psi[0], s->hsum[0], b);
    return s;
}

void xfp_destroy(xfp_sim* s)
{
    if (!s) return;
    for (int p = 0; p < 4; ++p) free(s->fq[p]);
    free(s->hvac);
    free(s->Cos2R); free(s->dCos2R); free(s->SinR); free(s->sinphi); free(s->cosphi);
    free(s->cosb); free(s->sinb); free(s->dcosb); free(s->dl);
    const int ids[4] = {0, 1, 3, 4};
    for (int k = 0; k < 4; ++k) { free(s->psi[ids[k]]); free(s->hsum[ids[k]]); }
    free(s);
}

int xfp_geometry(const xfp_sim* s) { return s->geom; }
int xfp_nbeams(const xfp_sim* s) { return s->nbeams; }
int xfp_ebins(const xfp_sim* s) { return s->ne; }
int xfp_abins(const xfp_sim* s) { return s->tet; }
int xfp_pbins(const xfp_sim* s) { return s->pb; }

void xfp_params(const xfp_sim* s, double out[10])
{
    out[0] = s->R0; out[1] = s->Rn; out[2] = s->dr0; out[3] = s->eps0; out[4] = s->ksi;
    out[5] = s->maxdr; out[6] = s->Ts; out[7] = s->Tn; out[8] = (double)s->seed; out[9] = s->noise_amp;
}

void xfp_tables(const xfp_sim* s, double* fv, double* hvac, double* LE, double* Ev)
{
    for (int p = 0; p < 4; ++p) memcpy(fv + p * s->ne, s->fq[p], s->ne * sizeof(double));
    memcpy(hvac, s->hvac, 2 * s->ne * sizeof(double));
    memcpy(LE, s->LE, 4 * sizeof(double));
    memcpy(Ev, s->Ev, 4 * sizeof(double));
}

static int role(const xfp_sim* s, int which)
{
    if (which == 0) return s->i0;
    if (which == 4) return s->i4;
    return which;
}

void xfp_set_state(xfp_sim* s, const double* psi)
{
    memcpy(s->psi[s->i0], psi, (size_t)s->nbeams * 4 * s->ne * sizeof(double));
#pragma omp parallel for
    for (int b = 0; b < s->nbeams; ++b) calc_esum(s, s->psi[s->i0], s->hsum[s->i0], b);
}

void xfp_get_state(const xfp_sim* s, int which, double* psi)
{
    memcpy(psi, s->psi[role(s, which)], (size_t)s->nbeams * 4 * s->ne * sizeof(double));
}

void xfp_get_esum(const xfp_sim* s, int which, double* out)
{
    memcpy(out, s->hsum[role(s, which)], (size_t)s->nbeams * 4 * sizeof(double));
}

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

/* Initial state of src/NBeam.cpp:260-275 with a seeded generator in place of rand(). */
void xfp_noise(xfp_sim* s, uint64_t seed, double amp)
{
    const int ne = s->ne;
    double* psi = s->psi[s->i0];
    for (int b = 0; b < s->nbeams; ++b) {
        int p = b % 4;
        for (int e = 0; e < ne; ++e) {
            double eps = (noise_u01(seed, b, e, 0) - 0.5) * amp;
            double eta = (noise_u01(seed, b, e, 1) - 0.5) * amp;
            double one_sq = sqrt(1. - eps * eps - eta * eta);
            BEAM(psi, b, 0)[e] = (p < 2) ? one_sq : eps;
            BEAM(psi, b, 1)[e] = 0.;
            BEAM(psi, b, 2)[e] = (p < 2) ? eps : one_sq;
            BEAM(psi, b, 3)[e] = eta;
        }
    }
#pragma omp parallel for
    for (int b = 0; b < s->nbeams; ++b) calc_esum(s, psi, s->hsum[s->i0], b);
}

static void geometry_for_step(xfp_sim* s, double r, double dr)
{
    double dr2 = .5 * dr;
    double rdr = r + dr;
    double rdr2 = r + dr2;
    calc_angle_bins(s, r, 0);
    calc_angle_bins(s, rdr2, 1);
    calc_angle_bins(s, rdr, 2);
    calc_delta_ls(s, dr2, 0, 0, 1);
    calc_delta_ls(s, dr, 1, 0, 2);
    calc_delta_ls(s, dr2, 2, 1, 2);
}

void xfp_probe(xfp_sim* s, double r, double dr, double* cosb, double* sinb, double* dcosb, double* dl)
{
    geometry_for_step(s, r, dr);
    const size_t n = (size_t)3 * s->tet * sizeof(double);
    memcpy(cosb, s->cosb, n);
    memcpy(sinb, s->sinb, n);
    memcpy(dcosb, s->dcosb, n);
    memcpy(dl, s->dl, n);
}

void xfp_calc_hvv(xfp_sim* s, int which, int pt, double* hvv)
{
    calc_hvv(s, s->hsum[role(s, which)], pt, hvv);
}

/* One iteration, src/Nmr.cpp:153-206. */
double xfp_iterate(xfp_sim* s, double r, double dr)
{
    const double rdr = r + dr, rdr2 = r + .5 * dr;
    double hm_r = xfp_hm(s, r), hm_rdr2 = xfp_hm(s, rdr2), hm_rdr = xfp_hm(s, rdr);
    geometry_for_step(s, r, dr);
    const size_t nh = (size_t)s->tet * s->pb * 4;
    double* h0 = (double*)xalloc(nh * sizeof(double));
    double* h1 = (double*)xalloc(nh * sizeof(double));
    double* h3 = (double*)xalloc(nh * sizeof(double));
    double* h4 = (double*)xalloc(nh * sizeof(double));
    double *b0 = s->psi[s->i0], *b1 = s->psi[1], *b3 = s->psi[3], *b4 = s->psi[s->i4];
    double *s0 = s->hsum[s->i0], *s1 = s->hsum[1], *s3 = s->hsum[3], *s4 = s->hsum[s->i4];
    calc_hvv(s, s0, 0, h0);                                 /* S1 */
    sweep(s, SW_HVV, 1, h0, hm_r, b0, b1, s1, NULL);        /* S2 */
    sweep(s, SW_HVV, 0, h0, hm_r, b0, b3, s3, NULL);        /* S6 */
    calc_hvv(s, s1, 2, h1);                                 /* S3 */
    sweep(s, SW_AVG, 1, h1, hm_rdr, b0, b4, NULL, b1);      /* S4/S5 */
    calc_hvv(s, s3, 1, h3);                                 /* S7 */
    sweep(s, SW_HVV, 1, h3, hm_rdr2, b0, b4, s4, NULL);     /* S8 */
    calc_hvv(s, s4, 2, h4);                                 /* S9 */
    sweep(s, SW_AVG_INPLACE, 2, h4, hm_rdr, NULL, b3, NULL, b4); /* S10/S11 */
    double max_err = -1.;
    const int NB = s->nbeams;
#pragma omp parallel for reduction(max : max_err)
    for (int i = 0; i < NB; ++i) {
        double e = calc_err_hvv(s, b4, b1, s4, i);
        max_err = (e > max_err) ? e : max_err;
    }
    free(h0); free(h1); free(h3); free(h4);
    return sqrt(max_err);
}

void xfp_accept(xfp_sim* s)
{
    int t = s->i0;
    s->i0 = s->i4;
    s->i4 = t;
}

long xfp_run(xfp_sim* s, double r, double dr, long max_iters, double* log, long log_cap, long* n_acc,
             double* r_end, double* dr_end)
{
    long Ts = max_iters >= 0 ? max_iters : s->Ts;
    long counter_tot = 0, counter = 0;
    time_t t0 = time(NULL);
    while (1) {
        int go = (r < s->Rn) && ((long)(time(NULL) - t0) < s->Tn) && (counter_tot < Ts);
        if (!go) break;
        double Max_err = xfp_iterate(s, r, dr);
        if (Max_err < s->eps0) {
            r += dr;
            xfp_accept(s);
            if (log && counter < log_cap) {
                log[3 * counter + 0] = (double)counter_tot;
                log[3 * counter + 1] = r;
                log[3 * counter + 2] = dr;
            }
            counter++;
        }
        counter_tot++;
        dr *= s->ksi * sqrt(s->eps0 / Max_err);
        dr = (dr > s->maxdr) ? s->maxdr : dr;
        dr = (r + dr > s->Rn) ? s->Rn - r : dr;
    }
    if (n_acc) *n_acc = counter;
    if (r_end) *r_end = r;
    if (dr_end) *dr_end = dr;
    return counter_tot;
}

void xfp_replay(xfp_sim* s, const double* r_before, const double* dr, long n)
{
    for (long i = 0; i < n; ++i) {
        (void)xfp_iterate(s, r_before[i], dr[i]);
        xfp_accept(s);
    }
}
