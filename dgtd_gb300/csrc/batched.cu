// Batched FP32 + 3xTF32 form (placeholder until the tensor-core kernels land).
#include <stdexcept>

#include "batched.hpp"

namespace dgtd {

std::unique_ptr<BatchedOp> BatchedOp::create(const RefTet&, const MeshTables&, const TablesDev&, int)
{
    throw std::runtime_error("the FP32 3xTF32 batched form is not available in this build");
}

}  // namespace dgtd
