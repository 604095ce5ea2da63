// TEST INFRASTRUCTURE: stands in for rtpslib/system/SPH.h when the
// reference's SPHSettings.cpp (SPH::calculate, SPH::updateParams) is compiled
// on its own.  build_ref.py copies SPHSettings.cpp into a scratch directory
// and writes this file beside it as SPH.h.  It declares the members those two
// functions use and nothing of the OpenCL system; the headers it includes are
// the reference's own, in the order that gives SPHSettings.cpp the same names
// (IV.h's `using namespace std;`, which makes log and pow the float
// overloads there as in the reference's build).
#pragma once
#define RTPS_UTIL_H_INCLUDED  // util.h includes the OpenCL headers
#include <cmath>
#include <iostream>

#include "debug.h"
#include "RTPSSettings.h"
#include "domain/Domain.h"
#include "domain/IV.h"
#include "system/SPHSettings.h"

namespace rtps {

// updateParams uploads the block with cl_sphp.copyToDevice(sphp)
struct ParamsUpload {
    void copyToDevice(const SPHParams&) {}
};

class SPH {
public:
    RTPSSettings* settings = nullptr;
    Domain grid;
    unsigned int max_num = 0;
    SPHParams sphp;
    ParamsUpload cl_sphp;
    void calculate();
    void updateParams();
};

}  // namespace rtps
