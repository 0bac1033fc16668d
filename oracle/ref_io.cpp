// Oracle harness (test infrastructure only; never part of the product path).
//
// Project-written replacement for the reference's NetCDF IO module, so that the
// reference's own hot-path sources (src/Nmr.cpp, src/Phy_MA.cpp, src/Phy_MAA.cpp,
// src/NBeam.cpp, ...) link without libnetcdf.  It implements the four entry
// points declared in include/Fio.h:22-38 (namespace nbgrp::io_f):
//   init, freemem, fillInitData, dumpToFile.
// Instead of writing files, dumpToFile records every accepted step
// (iteration index, radius after the step, dr used) and remembers the pointer
// to the accepted state, which ref_main.cpp writes out when the loop ends.
//
// The reference calls dumpToFile once per accepted step from
// src/Nmr.cpp:238 with (psi0_new, counter_tot, r_after, dr_used).
#include <vector>
#include <cstdio>

#include "global.h"
#include "NBeam.h"
#include "Fio.h"

namespace oracle_io {
std::vector<double> accepted;          // triples: itr, r, dr
const nbm::NBeam* last_state = 0;      // psi0 after the last accepted step
long n_accepted = 0;
}

namespace nbgrp {
namespace io_f {

void init(int) {}

void freemem() {}

void fillInitData(nbm::NBeam *REST) {}

void dumpToFile(const nbm::NBeam *REST nubeam, const int itr, const double r, const double dr, int, int) throw()
{
    oracle_io::accepted.push_back((double)itr);
    oracle_io::accepted.push_back(r);
    oracle_io::accepted.push_back(dr);
    oracle_io::last_state = nubeam;
    oracle_io::n_accepted++;
}

} // namespace io_f
} // namespace nbgrp
