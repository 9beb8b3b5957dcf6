// Single-instance FP32 stage on the tensor cores (single_tc.cu): work items of 8 elements,
// reference-element matrices as the A operand (streamed from a device image), fields and
// fluxes as the B operand, chain rule and curl in the epilogue.
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.hpp"
#include "refelem.hpp"

namespace dgtd {

bool tc1_supported(int p);
// A-operand image (uint32 words, tf32 hi/lo tiles) of Dr, Ds, Dt and LIFT in consumption order,
// repeated so that groups of CTAs stream different copies.
std::vector<uint32_t> tc1_operator_image(const RefTet& ref);
// One stage (A.mode) over all incidences; status: device flag set to 1 when a bounded wait gave up.
void launch_stage_tc1(const TablesF32& T, const StageArgsF32& A, const uint32_t* a_img, int* status, int n_sm,
                      cudaStream_t s);

}  // namespace dgtd
