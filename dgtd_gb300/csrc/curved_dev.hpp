// Second-order (curved) elements on the device: their block rows (curved.hpp) applied after
// each FP64 stage, with the stage's own register update.
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "curved.hpp"
#include "kernels.hpp"

namespace dgtd {

class CurvedOp {
public:
    // Builds the rows on the host and uploads them (blocks transposed for coalesced reads) with
    // the per-element flags the stage kernel skips.
    CurvedOp(const MeshTables& T, const RefTet& ref, double alpha);
    ~CurvedOp();
    CurvedOp(const CurvedOp&) = delete;
    CurvedOp& operator=(const CurvedOp&) = delete;

    const uint8_t* flags() const { return flags_; }
    int64_t n_elements() const { return n_; }
    int64_t device_bytes() const { return bytes_; }
    // dU/dt of the curved elements for the stage A (any mode), written as the stage kernel
    // writes its own elements.
    void apply(const TablesDev& T, const StageArgs& A, cudaStream_t s) const;

private:
    void release();
    int Np_ = 0;
    int64_t n_ = 0, bytes_ = 0;
    int32_t* elems_ = nullptr;
    int32_t* nbr_ = nullptr;
    double* blocks_ = nullptr;   // [n][5][col][row]
    uint8_t* flags_ = nullptr;   // [K]
};

}  // namespace dgtd
