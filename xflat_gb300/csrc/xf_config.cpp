// Config-file reader with the reference's key set, syntax and parse-time unit
// conversions (src/Parser.cpp:25-127): one "key= value" pair per line, '#'
// starts a comment line, unknown keys are skipped.  Extension keys used only by
// this implementation ("geometry=", "precision=", "seed=", "noise_amp=") are
// likewise skipped by the reference's parser, so one file serves both.
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "xf_physics.h"
#include "xflat_gpu.h"

extern "C" int xf_config_default(xf_config* c)
{
    if (!c) return XF_EINVAL;
    std::memset(c, 0, sizeof(*c));
    c->geometry = XF_GEOM_MA;
    c->precision = XF_PREC_FP64;
    c->abins = 0;
    c->pbins = 1;
    c->ebins = 0;
    c->flvs = 2;
    c->has_matter = 1;
    c->dump_mode = 0;
    c->Ts = 30000000;
    c->Tn = 10000000;
    c->new_file_step = 1000000;
    c->sync_step = 1000000;
    c->tstep1 = c->tstep2 = 300000;
    c->itrstep1 = c->itrstep2 = 3000000;
    c->start_beam = c->end_beam = -1;
    c->rstep1 = 10.;
    c->rstep2 = .5;
    c->eps0 = 1e-9;
    c->ksi = .94;
    c->R0 = 10.;
    c->Rn = 300.;
    c->dr = .001;
    c->max_dr = .1;
    c->Ye = .5;
    c->Rv = 10.;
    c->Mns = 1.4;
    c->gs = 0.7414067;
    c->S = 100.;
    c->hNS = .18;
    std::strcpy(c->file_prefix, "xflat");
    return XF_OK;
}

namespace {

template <typename T>
void rd(std::istringstream& ss, T& v)
{
    ss >> v;
}

int parse_stream(std::istream& in, xf_config* c)
{
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string k;
        ss >> k;
        if (k.empty() || k[0] == '#') continue;
        if (k == "filePrefix=") {
            std::string s;
            ss >> s;
            std::strncpy(c->file_prefix, s.c_str(), sizeof(c->file_prefix) - 1);
        }
        else if (k == "dumpMode=") rd(ss, c->dump_mode);
        else if (k == "newFile_step=") rd(ss, c->new_file_step);
        else if (k == "sync_step=") rd(ss, c->sync_step);
        else if (k == "r_step1=") rd(ss, c->rstep1);
        else if (k == "t_step1=") rd(ss, c->tstep1);
        else if (k == "itr_step1=") rd(ss, c->itrstep1);
        else if (k == "r_step2=") rd(ss, c->rstep2);
        else if (k == "t_step2=") rd(ss, c->tstep2);
        else if (k == "itr_step2=") rd(ss, c->itrstep2);
        else if (k == "start_beam=") rd(ss, c->start_beam);
        else if (k == "end_beam=") rd(ss, c->end_beam);
        else if (k == "hasMatter=") rd(ss, c->has_matter);
        else if (k == "eps0=") rd(ss, c->eps0);
        else if (k == "ksi=") rd(ss, c->ksi);
        else if (k == "mu=") rd(ss, c->mu);
        else if (k == "Tn=") rd(ss, c->Tn);
        else if (k == "Ts=") rd(ss, c->Ts);
        else if (k == "R0=") rd(ss, c->R0);
        else if (k == "Rn=") rd(ss, c->Rn);
        else if (k == "dr=") rd(ss, c->dr);
        else if (k == "max_dr=") rd(ss, c->max_dr);
        else if (k == "E0=") { rd(ss, c->E0); c->E0 *= xf::kMeV; }
        else if (k == "E1=") { rd(ss, c->E1); c->E1 *= xf::kMeV; }
        else if (k == "Pbins=") rd(ss, c->pbins);
        else if (k == "Abins=") rd(ss, c->abins);
        else if (k == "Ebins=") rd(ss, c->ebins);
        else if (k == "Flvs=") rd(ss, c->flvs);
        else if (k == "Ye=") rd(ss, c->Ye);
        else if (k == "Rv=") rd(ss, c->Rv);
        else if (k == "Mns=") rd(ss, c->Mns);
        else if (k == "gs=") rd(ss, c->gs);
        else if (k == "S=") rd(ss, c->S);
        else if (k == "hNS=") rd(ss, c->hNS);
        else if (k == "nb0=") { rd(ss, c->nb0); c->nb0 *= 1.E+15; }
        else if (k == "theta=") { rd(ss, c->theta); c->theta2 = c->theta * 2; }
        else if (k == "dm2=") { rd(ss, c->dm2); c->dm2 *= xf::kEV2; }
        else if (k == "Lve=") { rd(ss, c->Lv[0]); c->Lv[0] *= xf::kErgS; }
        else if (k == "Lv_e=") { rd(ss, c->Lv[1]); c->Lv[1] *= xf::kErgS; }
        else if (k == "Lvt=") { rd(ss, c->Lv[2]); c->Lv[2] *= xf::kErgS; }
        else if (k == "Lv_t=") { rd(ss, c->Lv[3]); c->Lv[3] *= xf::kErgS; }
        else if (k == "Tve=") { rd(ss, c->Tv[0]); c->Tv[0] *= xf::kMeV; }
        else if (k == "Tv_e=") { rd(ss, c->Tv[1]); c->Tv[1] *= xf::kMeV; }
        else if (k == "Tvt=") { rd(ss, c->Tv[2]); c->Tv[2] *= xf::kMeV; }
        else if (k == "Tv_t=") { rd(ss, c->Tv[3]); c->Tv[3] *= xf::kMeV; }
        else if (k == "eta_ve=") rd(ss, c->eta[0]);
        else if (k == "eta_v_e=") rd(ss, c->eta[1]);
        else if (k == "eta_vt=") rd(ss, c->eta[2]);
        else if (k == "eta_v_t=") rd(ss, c->eta[3]);
        else if (k == "geometry=") {
            std::string s;
            ss >> s;
            if (s == "MAA" || s == "maa") c->geometry = XF_GEOM_MAA;
            else if (s == "MA" || s == "ma") c->geometry = XF_GEOM_MA;
            else if (s == "SA" || s == "sa") c->geometry = XF_GEOM_SA;
            else return XF_EINVAL;
        }
        else if (k == "precision=") {
            std::string s;
            ss >> s;
            if (s == "fp64" || s == "FP64") c->precision = XF_PREC_FP64;
            else if (s == "mixed" || s == "MIXED") c->precision = XF_PREC_MIXED;
            else if (s == "df" || s == "DF") c->precision = XF_PREC_DF;
            else return XF_EINVAL;
        }
        else if (k == "seed=") { unsigned long long s = 0; ss >> s; c->seed = s; }
        else if (k == "noise_amp=") rd(ss, c->noise_amp);
    }
    return XF_OK;
}

}  // namespace

extern "C" int xf_config_parse(const char* text, xf_config* c)
{
    if (!text || !c) return XF_EINVAL;
    std::istringstream in(text);
    return parse_stream(in, c);
}

extern "C" int xf_config_load(const char* path, xf_config* c)
{
    if (!path || !c) return XF_EINVAL;
    std::ifstream in(path);
    if (!in.is_open()) return XF_EIO;
    return parse_stream(in, c);
}

extern "C" const char* xf_strerror(int s)
{
    switch (s) {
    case XF_OK: return "ok";
    case XF_EINVAL: return "invalid argument or configuration";
    case XF_ECUDA: return "CUDA error or no usable GPU";
    case XF_ETIMEOUT: return "bounded device wait timed out";
    case XF_ENAN: return "step error is NaN";
    case XF_EIO: return "file IO error";
    case XF_ENOMEM: return "out of memory";
    case XF_EUNSUPPORTED: return "unsupported option";
    default: return "unknown status";
    }
}
