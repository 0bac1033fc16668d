// Nmr_gpu.cpp -- the module a maintainer adds to XFLAT (as src/Nmr_gpu.cpp) to
// run the stepper loop on the GPU through libxflat_gb300.so.  It is compiled
// instead of src/Nmr.cpp and keeps namespace nbgrp::nmr's interface
// (include/Nmr.h:20-31: init, evolutionLoop, freemem, and the host beam array
// nubm_0 that the IO module reads); Parser, the NBGroup init order and the IO
// module stay as they are.
//
// Two forms of evolutionLoop:
//  - default: the loop runs under device control when nothing is written;
//    with dumpMode set it runs host-driven and XFLAT's own fio::dumpToFile
//    writes the files from a host copy of the state on every accepted step
//    (src/Nmr.cpp:238);
//  - -DXFLAT_GPU_LIBRARY_FILES: the library writes the same Snapshot and
//    Probability files itself (the dump triggers of src/IO_f.cpp:387-424
//    evaluated on the GPU, records staged on the device and written by a
//    background thread), with no per-step copy of the state.
#include "xflat_gpu.h"
#include "Util.h"
#include "NBeam.h"
#include "Fio.h"
#include "Phy.h"
#include <vector>
#include <cstdio>

namespace nbgrp { namespace nmr {
using namespace nbm;
static xf_handle* H = 0;
static int length = 0;
NBeam* nubm_0;                      // host copy for fio::dumpToFile / fillInitData

static void to_cfg(xf_config* c)    // Util:: values are already in internal units
{
    xf_config_default(c);
    // the modules' data dimensions: SA 4 (r, prtcl, comp, ebin), MA 5, MAA 6
    c->geometry = (phy::getDim() == 6) ? XF_GEOM_MAA : (phy::getDim() == 4) ? XF_GEOM_SA : XF_GEOM_MA;
    c->abins = Util::Abins(); c->pbins = Util::Pbins(); c->ebins = Util::Ebins(); c->flvs = Util::Flvs();
    c->has_matter = Util::hasMatter(); c->Ts = Util::Ts(); c->Tn = Util::Tn();
    c->eps0 = Util::eps0(); c->ksi = Util::ksi(); c->R0 = Util::R0(); c->Rn = Util::Rn();
    c->dr = Util::dr(); c->max_dr = Util::maxDr(); c->E0 = Util::E0(); c->E1 = Util::E1();
    c->Ye = Util::Ye(); c->Rv = Util::Rv(); c->Mns = Util::Mns(); c->gs = Util::gs(); c->S = Util::S();
    c->hNS = Util::hNS(); c->nb0 = Util::nb0(); c->theta = Util::theta(); c->theta2 = Util::theta2();
    c->dm2 = Util::dm2();
    for (int i = 0; i < 4; ++i) { c->Lv[i] = Lv(i); c->Tv[i] = Tv(i); c->eta[i] = eta(i); }
}

static std::vector<double> buf;
static void pull()                  // device psi0 -> host NBeam arrays
{
    xf_get_state(H, 0, buf.data());
    for (int i = 0; i < length; ++i)
        for (int c = 0; c < 4; ++c)
            std::copy(&buf[(i * 4 + c) * nbm_ebins], &buf[(i * 4 + c + 1) * nbm_ebins], nubm_0[i].psi(c));
}

static int on_accept(void*, long itr, double r, double dr)
{
    pull();                                     // only when the IO module will write (dumpMode != 0)
    fio::dumpToFile(nubm_0, (int)itr, r, dr);
    return 0;
}

int init(int len)
{
    length = len;
    posix_memalign((void**)&nubm_0, ALIGN_LEN, len * sizeof(NBeam));
    phy::initBeam(nubm_0);                      // pure states, or the resume file
    xf_config c; to_cfg(&c);
    if (xf_create(&c, &H) != XF_OK) { printf("xf_create failed\n"); return -1; }
    buf.resize((size_t)len * 4 * nbm_ebins);
    for (int i = 0; i < len; ++i)
        for (int k = 0; k < 4; ++k)
            std::copy(nubm_0[i].psi(k), nubm_0[i].psi(k) + nbm_ebins, &buf[(i * 4 + k) * nbm_ebins]);
    xf_set_state(H, buf.data());
    return 3;
}

#ifndef XFLAT_GPU_LIBRARY_FILES
int evolutionLoop() throw()
{
    xf_run_opts o; xf_run_opts_default(&o);
    o.device_control = Util::dumpMode() ? 0 : 1;   // no per-step host work when nothing is written
    xf_run_stats s;
    int rc = xf_run(H, &o, Util::dumpMode() ? on_accept : 0, 0, &s);
    if (rc != XF_OK) printf("xf_run: %s (%s)\n", xf_strerror(rc), xf_last_error(H));
    pull();
    printf("Total iterations: %ld\tCorrect iterations: %ld\t at radius(Km): %f\n", s.iterations, s.accepted, s.r_end);
    return (int)s.iterations;
}
#else
int evolutionLoop() throw()
{
    xf_run_opts o; xf_run_opts_default(&o);
    o.write_files = Util::dumpMode() ? 1 : 0;       // Snapshot/Probability files, asynchronous
    o.device_control = 1;                           // triggers evaluated and records staged on the GPU
    xf_run_stats s;
    int rc = xf_run(H, &o, 0, 0, &s);               // files complete and flushed on return
    if (rc != XF_OK) printf("xf_run: %s (%s)\n", xf_strerror(rc), xf_last_error(H));
    xf_io_close(H);
    pull();
    printf("Total iterations: %ld\tCorrect iterations: %ld\t at radius(Km): %f\n", s.iterations, s.accepted, s.r_end);
    return (int)s.iterations;
}
#endif

void freemem() { xf_destroy(H); phy::freeBeam(nubm_0); free(nubm_0); nbm::freemem(); }
}}
