// abi_internal.hpp -- the simulation context behind cmm_ctx, shared by the translation units
// that implement include/cmm_abi.h.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "settings.hpp"
#include "sim.hpp"

struct cmm_ctx {
    cmm::Settings settings;
    cmm::EulerSim* sim = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<double> discrete;
};

namespace cmm {
void set_last_error(const std::string& msg);
}
