// Batched FP32 + 3xTF32 form of the DG Maxwell step (B incidences per mesh).
#pragma once
#include <cstdint>
#include <memory>
#include <vector>

#include "kernels.hpp"
#include "mesh.hpp"
#include "refelem.hpp"

namespace dgtd {

class BatchedOp {
public:
    static std::unique_ptr<BatchedOp> create(const RefTet& ref, const MeshTables& mesh, const TablesDev& dev, int batch);
    virtual ~BatchedOp() = default;
    virtual void set_sources(const std::vector<PlaneWaveDev>& pw) = 0;
    virtual int64_t device_bytes() const = 0;
};

}  // namespace dgtd
