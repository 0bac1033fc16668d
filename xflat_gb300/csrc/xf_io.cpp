// Snapshot / Probability files and resume: the reference's NetCDF IO module
// (src/IO_f.cpp) on top of the project's classic-format writer and reader.
// Files, dimension and variable names, attribute names and values, dump
// triggers, file rotation and sync follow src/IO_f.cpp:90-424 so existing
// post-processing reads them unchanged.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "xf_engine.h"
#include "xf_netcdf.h"
#include "xf_physics.h"
#include "xflat_gpu.h"

struct xf_io {
    xf::nc::Writer snap, prob;
    int ctr = 0;               // files created so far (rotation counter)
    uint64_t itr = 0;          // records in the current snapshot file
    double last_r0 = 0., last_r1 = 0., last_r2 = 0.;
    long t1 = 0, t2 = 0;       // wall seconds of the last time-triggered dumps
    bool inited = false;
    int verbose = 0;
};

namespace {

long wall_s()
{
    return (long)std::chrono::duration_cast<std::chrono::seconds>(std::chrono::system_clock::now().time_since_epoch()).count();
}

std::string file_name(const xf_config& c, const char* kind, int ctr)
{
    // <prefix><kind><ctr>_<rank>_.nc with rank 0 (src/IO_f.cpp:119, 162)
    return std::string(c.file_prefix) + kind + std::to_string(ctr) + "_0_.nc";
}

// Dimensions, variables and attributes of the Snapshot file (src/IO_f.cpp:116-144);
// the dimensions are the module's getDimInfo/countDim: MA r, theta, prtcl,
// comp, ebin (src/Phy_MA.cpp), MAA adds phi (src/Phy_MAA.cpp), SA has no
// angle (src/Phy_SA.cpp:67-96).
void snapshot_schema(const xf_config& c, std::vector<xf::nc::Dim>& dims, std::vector<xf::nc::Var>& vars)
{
    using xf::nc::Attr;
    using xf::nc::Dim;
    using xf::nc::Var;
    int A, P;
    xf::beam_dims(c, A, P);
    dims.clear();
    dims.push_back(Dim{"r", 0});
    if (c.geometry != XF_GEOM_SA) dims.push_back(Dim{"theta", (uint64_t)A});
    if (c.geometry == XF_GEOM_MAA) dims.push_back(Dim{"phi", (uint64_t)P});
    dims.push_back(Dim{"prtcl", 4});
    dims.push_back(Dim{"comp", 4});
    dims.push_back(Dim{"ebin", (uint64_t)c.ebins});
    Var r{"r", {0}, {}}, dr{"dr", {0}, {}}, psi{"psi", {}, {}};
    for (int i = 0; i < (int)dims.size(); ++i) psi.dims.push_back(i);
    psi.atts.push_back(Attr{"E0", {c.E0}});
    psi.atts.push_back(Attr{"E1", {c.E1}});
    // src/IO_f.cpp:136-143 names the attributes string("..."+i): the literal
    // advanced by i characters, with the values Tv(i), Tv(i+1), eta(i),
    // eta(i+1).  Kept as written so readers of existing files match.
    const char* tp = "Teprature for particle";
    const char* ta = "Teprature for anti-particle";
    const char* ep = "eta for particle";
    const char* ea = "eta for anti-particle";
    for (int i = 0; i < c.flvs; ++i) {
        psi.atts.push_back(Attr{tp + i, {c.Tv[i]}});
        psi.atts.push_back(Attr{ta + i, {c.Tv[i + 1]}});
        psi.atts.push_back(Attr{ep + i, {c.eta[i]}});
        psi.atts.push_back(Attr{ea + i, {c.eta[i + 1]}});
    }
    vars = {r, dr, psi};
}

// io_f::init (src/IO_f.cpp:90-194)
int io_init(xf_handle* h, int ctr)
{
    xf_io& io = *h->io;
    const xf_config& c = h->cfg;
    io.ctr = ctr;
    io.itr = 0;
    io.last_r0 = c.R0;
    using xf::nc::Attr;
    using xf::nc::Dim;
    using xf::nc::Var;
    if (c.dump_mode & 1) {
        std::vector<Dim> dims;
        std::vector<Var> vars;
        snapshot_schema(c, dims, vars);
        if (!io.snap.create(file_name(c, "Snapshot", ctr), dims, vars))
            return h->fail(XF_EIO, "cannot create " + file_name(c, "Snapshot", ctr));
        io.last_r1 = c.R0;
        io.t1 = wall_s();
    }
    if (c.dump_mode & 2) {
        std::vector<Dim> dims = {Dim{"r", 0}, Dim{"theta", (uint64_t)h->A}, Dim{"phi", (uint64_t)h->P}};
        std::vector<Var> vars = {Var{"r", {0}, {}}};
        for (int p = 0; p < 4; ++p) vars.push_back(Var{"prtcl" + std::to_string(p), {0, 1, 2}, {}});
        if (!io.prob.create(file_name(c, "Probability", ctr), dims, vars))
            return h->fail(XF_EIO, "cannot create " + file_name(c, "Probability", ctr));
        io.last_r2 = c.R0;
        io.t2 = wall_s();
    }
    io.inited = true;
    return XF_OK;
}

void io_free(xf_io& io)
{
    io.snap.close();
    io.prob.close();
    io.inited = false;
}

// io_f::writeToFile for the snapshot (src/IO_f.cpp:266-328)
int write_snapshot(xf_handle* h, double r, double dr)
{
    xf_io& io = *h->io;
    const xf_config& c = h->cfg;
    if ((int64_t)io.itr >= c.new_file_step) {
        io.snap.close();
        io.prob.close();
        int rc = io_init(h, io.ctr + 1);
        if (rc) return rc;
    }
    std::vector<double> psi((size_t)h->nbeams * 4 * h->ne);
    int rc = h->get_state(0, psi.data());
    if (rc) return rc;
    if (!io.snap.append({&r, &dr, psi.data()})) return h->fail(XF_EIO, "snapshot write failed");
    io.itr++;
    if (c.sync_step > 0 && io.itr % c.sync_step == 0) io.snap.sync();
    return XF_OK;
}

// io_f::writeToFile for the probability file (src/IO_f.cpp:331-384)
int write_probability(xf_handle* h, double r)
{
    xf_io& io = *h->io;
    const int n = h->A * h->P;
    std::vector<double> sv((size_t)n * 4);
    int rc = xf_survival(h, sv.data());
    if (rc) return rc;
    std::vector<std::vector<double>> cols(4, std::vector<double>((size_t)n));
    for (int i = 0; i < n; ++i)
        for (int p = 0; p < 4; ++p) cols[p][i] = sv[(size_t)i * 4 + p];
    if (!io.prob.append({&r, cols[0].data(), cols[1].data(), cols[2].data(), cols[3].data()}))
        return h->fail(XF_EIO, "probability write failed");
    if (h->cfg.sync_step > 0 && io.itr % h->cfg.sync_step == 0) io.prob.sync();
    return XF_OK;
}

}  // namespace

int xf_handle::dump_files(long it, double r, double dr) { return xf_dump(this, it, r, dr); }

extern "C" {

// io_f::dumpToFile (src/IO_f.cpp:387-424)
int xf_dump(xf_handle* h, long it, double r, double dr)
{
    if (!h) return XF_EINVAL;
    if (!h->io) h->io = new xf_io();
    xf_io& io = *h->io;
    const xf_config& c = h->cfg;
    int rc;
    if (!io.inited && (rc = io_init(h, 0))) return rc;
    const long now = wall_s();
    if (!c.dump_mode) {
        if (r - io.last_r0 > 1.0) {
            io.last_r0 = r;
            if (io.verbose) std::printf("%f\n", r);
        }
    }
    if (c.dump_mode & 1) {
        if (r == c.Rn || r - io.last_r1 > c.rstep1 || (now - io.t1) > c.tstep1 || (c.itrstep1 > 0 && !(it % c.itrstep1))) {
            if (io.verbose) std::printf("%f\n", r);
            io.last_r1 = r;
            io.t1 = now;
            if ((rc = write_snapshot(h, r, dr))) return rc;
        }
    }
    if (c.dump_mode & 2) {
        if (r == c.Rn || r - io.last_r2 > c.rstep2 || (now - io.t2) > c.tstep2 || (c.itrstep2 > 0 && !(it % c.itrstep2))) {
            if (io.verbose) std::printf("%f\n", r);
            io.last_r2 = r;
            io.t2 = now;
            if ((rc = write_probability(h, r))) return rc;
        }
    }
    return XF_OK;
}

int xf_snapshot_write(const char* path, const xf_config* c, long nrec, const double* r, const double* dr,
                      const double* psi)
{
    int A = 0, P = 0;
    if (c) xf::beam_dims(*c, A, P);
    if (!path || !c || nrec < 0 || (nrec > 0 && (!r || !dr || !psi)) || A <= 0 || P <= 0 || c->ebins <= 0)
        return XF_EINVAL;
    std::vector<xf::nc::Dim> dims;
    std::vector<xf::nc::Var> vars;
    snapshot_schema(*c, dims, vars);
    xf::nc::Writer w;
    if (!w.create(path, dims, vars)) return XF_EIO;
    const size_t n = (size_t)A * P * 4 * 4 * c->ebins;
    for (long i = 0; i < nrec; ++i)
        if (!w.append({&r[i], &dr[i], psi + (size_t)i * n})) return XF_EIO;
    w.close();
    return XF_OK;
}

int xf_snapshot_read(const char* path, long rec, double* r, double* dr, double* psi, long* nrec)
{
    if (!path) return XF_EINVAL;
    xf::nc::Reader rd;
    if (!rd.open(path)) return XF_EIO;
    const int vpsi = rd.find_var("psi"), vr = rd.find_var("r"), vdr = rd.find_var("dr");
    if (vpsi < 0 || vr < 0 || vdr < 0) return XF_EIO;
    if (nrec) *nrec = (long)rd.records();
    if (rd.records() == 0) return (r || dr || psi) ? XF_EIO : XF_OK;
    const uint64_t k = rec < 0 ? rd.records() - 1 : (uint64_t)rec;
    if (k >= rd.records()) return XF_EINVAL;
    std::vector<double> v;
    if (r) {
        if (!rd.read(vr, k, v)) return XF_EIO;
        *r = v[0];
    }
    if (dr) {
        if (!rd.read(vdr, k, v)) return XF_EIO;
        *dr = v[0];
    }
    if (psi) {
        if (!rd.read(vpsi, k, v)) return XF_EIO;
        std::memcpy(psi, v.data(), v.size() * sizeof(double));
    }
    return XF_OK;
}

int xf_io_close(xf_handle* h)
{
    if (!h) return XF_EINVAL;
    if (h->io) {
        io_free(*h->io);
        delete h->io;
        h->io = nullptr;
    }
    return XF_OK;
}

int xf_io_verbose(xf_handle* h, int on)
{
    if (!h) return XF_EINVAL;
    if (!h->io) h->io = new xf_io();
    h->io->verbose = on;
    return XF_OK;
}

// io_f::fillInitData (src/IO_f.cpp:197-250): the last record of psi, r and dr.
int xf_resume(xf_handle* h, const char* path, double* r, double* dr)
{
    if (!h || !path) return XF_EINVAL;
    xf::nc::Reader rd;
    if (!rd.open(path)) return h->fail(XF_EIO, std::string("cannot read NetCDF file ") + path);
    const int vpsi = rd.find_var("psi"), vr = rd.find_var("r"), vdr = rd.find_var("dr");
    if (vpsi < 0 || vr < 0 || vdr < 0 || rd.records() == 0)
        return h->fail(XF_EIO, std::string("no psi/r/dr records in ") + path);
    if (rd.count(vpsi) != (uint64_t)h->nbeams * 4 * h->ne)
        return h->fail(XF_EINVAL, std::string("psi in ") + path + " does not match this configuration's shape");
    const uint64_t last = rd.records() - 1;
    std::vector<double> psi, rv, drv;
    if (!rd.read(vpsi, last, psi) || !rd.read(vr, last, rv) || !rd.read(vdr, last, drv))
        return h->fail(XF_EIO, std::string("short read from ") + path);
    int rc = h->set_state(psi.data());
    if (rc) return rc;
    if (r) *r = rv[0];
    if (dr) *dr = drv[0];
    return XF_OK;
}

}  // extern "C"
