// des_mixed.cuh -- launchers of the mixed-precision (DES_PREC_MIXED) kernels.
#pragma once

#include <cuda_runtime.h>

#include "des_common.cuh"

namespace des {

int launch_update_stress_mixed(const KP &p, cudaStream_t s, bool fused);
int launch_strain_rate_mixed(const KP &p, cudaStream_t s, bool begin_step);
int launch_heat_and_dvoldt_mixed(const KP &p, cudaStream_t s, bool heat, bool dvoldt);
// fused step: strain rate + heat terms + dvoldt terms, then the nodal sums and the temperature update
int launch_elem_pass_mixed(const KP &p, cudaStream_t s, bool heat);
// mass_sums: first the compute_mass sums of the look-ahead geometry pass's
// element terms (k_mass_sum's); begin_step: advance the clock (steps, time)
int launch_node_pass_mixed(const KP &p, cudaStream_t s, bool heat, bool mass_sums = false, bool begin_step = false);

}  // namespace des
