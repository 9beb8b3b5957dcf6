// Thin-layer boundaries (SGBC) on the device: per-pair sub-solver states and the kernels that
// couple them to the FP64 stage (sgbc.cu). Host tables come from sgbc.hpp.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.hpp"
#include "sgbc.hpp"

namespace dgtd {

constexpr int kSgbcMaxStacks = 16;

class SgbcOp {
public:
    // Builds the sub-solvers and the pair layout and allocates the device state (zero fields).
    // alpha: the operator's upwind coefficient (the injection flux of curved elements' SGBC faces)
    SgbcOp(const MeshTables& T, const RefTet& ref, const std::vector<SgbcStackSpec>& stacks,
           const std::vector<int32_t>& face_stack, double alpha);
    ~SgbcOp();
    SgbcOp(const SgbcOp&) = delete;
    SgbcOp& operator=(const SgbcOp&) = delete;

    int64_t n_pairs() const { return static_cast<int64_t>(layout_.gl.size()); }
    int n_stacks() const { return static_cast<int>(stacks_.size()); }
    const SgbcStack1D& stack(int i) const { return stacks_[i]; }

    // The step's checkpoint (GlobalEvolution::commitSGBCCheckpoint): the current states become
    // the checkpoint every stage restarts from, t the start time, dt the step, and the face-frame
    // ghost values of x (the step's start state) are kept for the finalisation.
    void commit(const TablesDev& T, const double* x, double t, double dt, cudaStream_t s);
    // The step's end (GlobalEvolution::finalizeSGBCStep): the states advance from the checkpoint
    // over dt with ghosts interpolated between the checkpoint's and x's (the step's end state).
    void finalize(const TablesDev& T, const double* x, cudaStream_t s);

    // Before a stage on input `in` at stage time t (MODE_MULT: span t - base; RK4 stage k: the
    // nominal span c_k dt, sub-step count from t - base). RK4 stage 1 commits the checkpoint.
    void before_stage(const TablesDev& T, const StageArgs& A, double t, cudaStream_t s);
    // After the stage kernel: adds the SGBC face flux into the stage's outputs; after RK4 stage 4
    // finalises the step.
    void after_stage(const TablesDev& T, const StageArgs& A, cudaStream_t s);

    // Copies of the current per-pair states (tests): [pairs][n of the pair's stack] concatenated.
    void read_states(double* host) const;
    int64_t state_len() const { return state_len_; }
    double base_time() const { return base_; }
    int64_t launches() const { return launches_; }

private:
    struct DevMap {
        double* a = nullptr;   // stage: R then G; final: FT then Vo then Vn
        int64_t n = 0;
    };
    const DevMap& stage_map(int st, double span, int nsteps);
    void release();
    void trim_maps();
    const DevMap& final_map(int st, double span, int nsteps);

    std::vector<SgbcStack1D> stacks_;
    SgbcLayout layout_;
    int64_t state_len_ = 0;
    double base_ = 0.0;
    double step_dt_ = 0.0;
    int64_t launches_ = 0;
    std::map<std::tuple<int, int, double, int>, DevMap> maps_;   // (kind, stack, span, nsteps)
    // device buffers
    int32_t *gl_ = nullptr, *gr_ = nullptr, *pstack_ = nullptr;
    double* rot_ = nullptr;
    int64_t* xoff_ = nullptr;
    // states and their norms, double-buffered: [cp_] is the checkpoint every stage restarts from,
    // [cur_] the current states (the finalisation writes the buffer that is not the checkpoint)
    double* X_[2] = {nullptr, nullptr};
    double* snorm_[2] = {nullptr, nullptr};
    int cp_ = 0, cur_ = 0;
    double* gold_ = nullptr;
    double* gnew_ = nullptr;
    double* trace_ = nullptr;
    int* flags_ = nullptr;   // [8]: per-stage quiescence flags (0 all quiescent), slot 7 finalisation
    int32_t *el_elem_ = nullptr, *el_start_ = nullptr, *ent_face_ = nullptr, *ent_role_ = nullptr, *ent_pairs_ = nullptr;
    // SGBC faces of curved elements: per entry the offset of its dense injection blocks (Bm then
    // Bp, transposed) in cblk_, or -1 for a straight element's face
    int64_t* ent_cblk_ = nullptr;
    double* cblk_ = nullptr;
    size_t flux_shmem_ = 0;
    int cur_flag_ = 0;
};

}  // namespace dgtd
