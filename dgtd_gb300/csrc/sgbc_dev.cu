// Thin-layer boundaries (SGBC) on the device.
//
// Per RK stage (reference GlobalEvolution::Mult, src/evolution/GlobalEvolution.cpp:639-1001):
//  - sgbc_trace: per face node pair, the stage input at its two nodes rotated to the face frame
//    (ghost data), the quiescence tests (state and interface below 1e-8), and the slab's interface
//    values after the advance from the checkpoint to the stage time: R x_cp + G g with the
//    stack's composed sub-step maps; rotated back, or the stack's PEC/PMC/SMA mirror, they are
//    the neighbour traces of the two 3D elements;
//  - the FP64 stage kernel gives SGBC faces no flux (the reference leaves them out of the
//    interior flux);
//  - sgbc_flux: per element with SGBC faces, the interior upwind flux with those traces, lifted
//    and scaled like the stage kernel's, added into the stage's outputs with the RK4 register
//    coefficients (the injection is linear in the flux).
// After RK4 stage 4 (GlobalEvolution::finalizeSGBCStep, GlobalEvolution.cpp:433-545):
//  - sgbc_quiesce: ghost values of the new state and the all-quiescent test;
//  - sgbc_final: per pair x = F x_cp + Vo g_old + Vn g_new (the advance over the whole step with
//    interpolated ghosts) and the new state's norm for the next step's quiescence tests.
// Every kernel indexes only the pairs, entries and stacks the host built and checked.
#include "sgbc_dev.hpp"

#include "curved.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <stdexcept>
#include <string>

namespace dgtd {

namespace {

constexpr double kQuiet = 1e-8;   // the reference's sgbc_skip_threshold_ (GlobalEvolution.h:92-95)

struct StackInfo {
    int64_t n, local, idx_left, idx_right;
    int left_bc, right_bc;
    const double* R;    // stage map [12][n]
    const double* G;    // stage map [12][12]
    const double* FT;   // final map [n][n] transposed
    const double* Vo;   // [n][12]
    const double* Vn;   // [n][12]
};

struct PairArgs {
    int64_t n_pairs;
    int64_t N;
    const int32_t* gl;
    const int32_t* gr;
    const int32_t* pstack;
    const double* rot;
    const int64_t* xoff;
    const double* X;       // checkpoint states
    const double* snorm;   // their norms
    double* Xout;          // finalisation: the new states
    double* snorm_out;     // and their norms
    double* gold;
    double* gnew;
    double* trace;
    int* flag;
    int n_stacks;
    StackInfo st[kSgbcMaxStacks];
};

__device__ __forceinline__ void to_local(const double* R, const double* u, double* g)
{
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        g[i] = R[3 * i] * u[0] + R[3 * i + 1] * u[1] + R[3 * i + 2] * u[2];
        g[3 + i] = R[3 * i] * u[3] + R[3 * i + 1] * u[4] + R[3 * i + 2] * u[5];
    }
}

__device__ __forceinline__ void to_global(const double* R, const double* v, double* u)
{
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        u[d] = R[d] * v[0] + R[3 + d] * v[1] + R[6 + d] * v[2];
        u[3 + d] = R[d] * v[3] + R[3 + d] * v[4] + R[6 + d] * v[5];
    }
}

// the slot value of a stack side closed by a sheet (fillBCSlot, GlobalEvolution.cpp:839-871)
__device__ __forceinline__ void mirror(int bc, const double* u, double* out)
{
    const double se = (bc == 1) ? -1.0 : 1.0, sh = (bc == 2) ? -1.0 : 1.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) { out[d] = se * u[d]; out[3 + d] = sh * u[3 + d]; }
}

// one warp per pair
__global__ void __launch_bounds__(256) sgbc_trace_kernel(PairArgs A, const double* __restrict__ in, int advance,
                                                        int store_old)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t p = warp; p < A.n_pairs; p += nwarps) {
        const StackInfo& S = A.st[A.pstack[p]];
        const int64_t gl = A.gl[p], gr = A.gr[p];
        double ug[12];
#pragma unroll
        for (int c = 0; c < 6; ++c) { ug[c] = in[c * A.N + gl]; ug[6 + c] = in[c * A.N + gr]; }
        double if2 = 0.0;
#pragma unroll
        for (int c = 0; c < 12; ++c) if2 += ug[c] * ug[c];
        const double* R9 = A.rot + p * 9;
        double g[12];
        to_local(R9, ug, g);
        to_local(R9, ug + 6, g + 6);
        const bool active = (A.snorm[p] >= kQuiet) || (if2 >= kQuiet * kQuiet);
        const double* x = A.X + A.xoff[p];
        double out[12];
        if (advance && active) {   // warp-uniform
            double acc[12];
#pragma unroll
            for (int r = 0; r < 12; ++r) acc[r] = 0.0;
            for (int64_t j = lane; j < S.n; j += 32) {
                const double xj = x[j];
#pragma unroll
                for (int r = 0; r < 12; ++r) acc[r] = fma(S.R[r * S.n + j], xj, acc[r]);
            }
#pragma unroll
            for (int r = 0; r < 12; ++r) {
                double v = acc[r];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                double gg = 0.0;
#pragma unroll
                for (int c = 0; c < 12; ++c) gg = fma(S.G[r * 12 + c], g[c], gg);
                out[r] = v + gg;
            }
        } else {
#pragma unroll
            for (int r = 0; r < 12; ++r) out[r] = x[(r % 6) * S.local + (r < 6 ? S.idx_left : S.idx_right)];
        }
        if (lane == 0) {
            if (active) atomicOr(A.flag, 1);
            if (store_old)
                for (int r = 0; r < 12; ++r) A.gold[p * 12 + r] = g[r];
            double* tr = A.trace + p * 12;
            double v[6];
            if (S.left_bc) mirror(S.left_bc, ug, v); else to_global(R9, out, v);
            for (int c = 0; c < 6; ++c) tr[c] = v[c];
            if (S.right_bc) mirror(S.right_bc, ug + 6, v); else to_global(R9, out + 6, v);
            for (int c = 0; c < 6; ++c) tr[6 + c] = v[c];
        }
    }
}

struct FluxArgs {
    const double* in;
    const double* trace;
    const int* flag;
    int64_t n_elems;
    const int32_t* el_elem;
    const int32_t* el_start;
    const int32_t* ent_face;
    const int32_t* ent_role;
    const int32_t* ent_pairs;
    const int64_t* ent_cblk;
    const double* cblk;
    int mode;
    double dt;
    double* out;
    double* yout;
    double* z;
    double* x;
};

__device__ __forceinline__ void sgbc_add(const FluxArgs& A, int64_t o, double ks)
{
    const double dt = A.dt;
    switch (A.mode) {
    case MODE_MULT: A.out[o] += ks; break;
    case MODE_RK4_1: A.yout[o] += 0.5 * dt * ks; A.z[o] += (dt / 6.0) * ks; break;
    case MODE_RK4_2: A.yout[o] += 0.5 * dt * ks; A.z[o] += (dt / 3.0) * ks; break;
    case MODE_RK4_3: A.yout[o] += dt * ks; A.z[o] += (dt / 3.0) * ks; break;
    case MODE_RK4_4: A.x[o] += (dt / 6.0) * ks; break;
    default: break;
    }
}

// one block per element with SGBC faces (at most 4 entries: one per face)
__global__ void __launch_bounds__(128) sgbc_flux_kernel(TablesDev T, FluxArgs A)
{
    if (*A.flag == 0) return;   // every pair quiescent: no injection
    extern __shared__ double sfl[];   // straight: [4][Nfp][6]; curved: [6 Np] state, [4][6][Nfp] traces
    const int Np = T.Np, Nfp = T.Nfp;
    const int64_t N = T.N;
    for (int64_t ie = blockIdx.x; ie < A.n_elems; ie += gridDim.x) {
        const int64_t e = A.el_elem[ie];
        const int k0 = A.el_start[ie], nent = A.el_start[ie + 1] - k0;
        if (A.ent_cblk[k0] >= 0) {   // a curved element: its dense injection blocks
            const int R = 6 * Np, F6 = 6 * Nfp;
            double* su = sfl;
            double* st = sfl + R;
            for (int w = threadIdx.x; w < R; w += blockDim.x) {
                const int c = w / Np, i = w - c * Np;
                su[w] = A.in[c * N + e * Np + i];
            }
            for (int w = threadIdx.x; w < nent * F6; w += blockDim.x) {
                const int k = w / F6, rr = w - k * F6, c = rr / Nfp, a = rr - c * Nfp;
                const int64_t pr = A.ent_pairs[static_cast<int64_t>(k0 + k) * Nfp + a];
                st[w] = A.trace[pr * 12 + A.ent_role[k0 + k] * 6 + c];
            }
            __syncthreads();
            for (int r = threadIdx.x; r < R; r += blockDim.x) {
                double acc = 0.0;
                for (int k = 0; k < nent; ++k) {
                    const double* BmT = A.cblk + A.ent_cblk[k0 + k];
                    const double* BpT = BmT + static_cast<size_t>(R) * R;
                    for (int col = 0; col < R; ++col) acc = fma(BmT[static_cast<size_t>(col) * R + r], su[col], acc);
                    for (int col = 0; col < F6; ++col) acc = fma(BpT[static_cast<size_t>(col) * R + r], st[k * F6 + col], acc);
                }
                const int c = r / Np, i = r - c * Np;
                sgbc_add(A, c * N + e * Np + i, acc);
            }
            __syncthreads();
            continue;
        }
        for (int w = threadIdx.x; w < nent * Nfp; w += blockDim.x) {
            const int k = w / Nfp, a = w - k * Nfp;
            const int ent = k0 + k;
            const int f = A.ent_face[ent], role = A.ent_role[ent];
            const int64_t pr = A.ent_pairs[static_cast<int64_t>(ent) * Nfp + a];
            const int vm = T.Fmask[f * Nfp + a];
            const double* fg = T.fgeo + e * 16 + f * 4;
            const double nx = fg[0], ny = fg[1], nz = fg[2], fs = fg[3];
            const double* uP = A.trace + pr * 12 + role * 6;
            double dE[3], dH[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                dE[c] = uP[c] - A.in[c * N + e * Np + vm];
                dH[c] = uP[c + 3] - A.in[(c + 3) * N + e * Np + vm];
            }
            const double aE = T.alpha, aH = T.alpha;
            const double ndE = nx * dE[0] + ny * dE[1] + nz * dE[2];
            const double ndH = nx * dH[0] + ny * dH[1] + nz * dH[2];
            const double h = 0.5 * fs;
            double* so = sfl + (k * Nfp + a) * 6;
            so[0] = h * ((ny * dH[2] - nz * dH[1]) + aE * (dE[0] - ndE * nx));
            so[1] = h * ((nz * dH[0] - nx * dH[2]) + aE * (dE[1] - ndE * ny));
            so[2] = h * ((nx * dH[1] - ny * dH[0]) + aE * (dE[2] - ndE * nz));
            so[3] = h * (-(ny * dE[2] - nz * dE[1]) + aH * (dH[0] - ndH * nx));
            so[4] = h * (-(nz * dE[0] - nx * dE[2]) + aH * (dH[1] - ndH * ny));
            so[5] = h * (-(nx * dE[1] - ny * dE[0]) + aH * (dH[2] - ndH * nz));
        }
        __syncthreads();
        const double ie_ = T.mat[e * 3 + 0], im_ = T.mat[e * 3 + 1];
        for (int i = threadIdx.x; i < Np; i += blockDim.x) {
            double lf[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            for (int k = 0; k < nent; ++k) {
                const int f = A.ent_face[k0 + k];
                for (int a = 0; a < Nfp; ++a) {
                    const double L = T.LIFTT[static_cast<int64_t>(f * Nfp + a) * Np + i];
                    const double* so = sfl + (k * Nfp + a) * 6;
#pragma unroll
                    for (int c = 0; c < 6; ++c) lf[c] = fma(L, so[c], lf[c]);
                }
            }
            const int64_t base = e * Np + i;
#pragma unroll
            for (int c = 0; c < 6; ++c) sgbc_add(A, base + c * N, (c < 3 ? ie_ : im_) * lf[c]);
        }
        __syncthreads();
    }
}

// one thread per pair: ghost values of the step's end state and the all-quiescent test
__global__ void __launch_bounds__(256) sgbc_quiesce_kernel(PairArgs A, const double* __restrict__ x_new)
{
    const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= A.n_pairs) return;
    const int64_t gl = A.gl[p], gr = A.gr[p];
    double ug[12];
    for (int c = 0; c < 6; ++c) { ug[c] = x_new[c * A.N + gl]; ug[6 + c] = x_new[c * A.N + gr]; }
    double if2 = 0.0;
    for (int c = 0; c < 12; ++c) if2 += ug[c] * ug[c];
    double g[12];
    to_local(A.rot + p * 9, ug, g);
    to_local(A.rot + p * 9, ug + 6, g + 6);
    for (int c = 0; c < 12; ++c) A.gnew[p * 12 + c] = g[c];
    if (A.snorm[p] >= kQuiet || if2 >= kQuiet * kQuiet) atomicOr(A.flag, 1);
}

// one block per pair: x = F x_cp + Vo g_old + Vn g_new, and |x|; every pair quiescent: the
// states stay at the checkpoint (copied)
__global__ void __launch_bounds__(256) sgbc_final_kernel(PairArgs A, int64_t n_max)
{
    const bool advance = *A.flag != 0;
    extern __shared__ double sx[];   // [n_max] state, then [24] ghosts
    __shared__ double red[256];
    double* gg = sx + n_max;
    for (int64_t p = blockIdx.x; p < A.n_pairs; p += gridDim.x) {
        const StackInfo& S = A.st[A.pstack[p]];
        const int64_t n = S.n;
        const double* x = A.X + A.xoff[p];
        double* xo = A.Xout + A.xoff[p];
        if (!advance) {
            for (int64_t j = threadIdx.x; j < n; j += blockDim.x) xo[j] = x[j];
            if (threadIdx.x == 0) A.snorm_out[p] = A.snorm[p];
            continue;
        }
        for (int64_t j = threadIdx.x; j < n; j += blockDim.x) sx[j] = x[j];
        if (threadIdx.x < 24)
            gg[threadIdx.x] = (threadIdx.x < 12) ? A.gold[p * 12 + threadIdx.x] : A.gnew[p * 12 + threadIdx.x - 12];
        __syncthreads();
        double ss = 0.0;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
            double acc = 0.0;
            for (int64_t j = 0; j < n; ++j) acc = fma(S.FT[j * n + i], sx[j], acc);
#pragma unroll
            for (int c = 0; c < 12; ++c) {
                acc = fma(S.Vo[i * 12 + c], gg[c], acc);
                acc = fma(S.Vn[i * 12 + c], gg[12 + c], acc);
            }
            xo[i] = acc;
            ss += acc * acc;
        }
        red[threadIdx.x] = ss;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) A.snorm_out[p] = sqrt(red[0]);
        __syncthreads();
    }
}

void ckd(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
T* upload(const std::vector<T>& v)
{
    T* d = nullptr;
    const size_t bytes = std::max<size_t>(1, v.size()) * sizeof(T);
    ckd(cudaMalloc(&d, bytes), "cudaMalloc SGBC table");
    if (!v.empty()) {
        cudaError_t e = cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { cudaFree(d); ckd(e, "cudaMemcpy SGBC table"); }
    }
    return d;
}

template <typename T>
T* zeros(size_t count)
{
    T* d = nullptr;
    ckd(cudaMalloc(&d, std::max<size_t>(1, count) * sizeof(T)), "cudaMalloc SGBC state");
    cudaError_t e = cudaMemset(d, 0, std::max<size_t>(1, count) * sizeof(T));
    if (e != cudaSuccess) { cudaFree(d); ckd(e, "cudaMemset SGBC state"); }
    return d;
}

constexpr int kGridCap = 4 * 152;

}  // namespace

SgbcOp::SgbcOp(const MeshTables& T, const RefTet& ref, const std::vector<SgbcStackSpec>& stacks,
               const std::vector<int32_t>& face_stack, double alpha)
{
    if (stacks.empty()) throw std::invalid_argument("SGBC: at least one stack is needed");
    if (static_cast<int>(stacks.size()) > kSgbcMaxStacks)
        throw std::invalid_argument("SGBC: at most " + std::to_string(kSgbcMaxStacks) + " stacks per operator");
    for (const auto& sp : stacks) stacks_.push_back(build_sgbc_stack(sp));
    layout_ = build_sgbc_layout(T, ref, face_stack, static_cast<int>(stacks_.size()));
    std::vector<int64_t> xoff(layout_.gl.size());
    int64_t off = 0;
    for (size_t p = 0; p < layout_.gl.size(); ++p) {
        xoff[p] = off;
        off += stacks_[layout_.stack[p]].n;
    }
    state_len_ = off;
    const size_t np = layout_.gl.size();
    // every index the kernels follow, checked once here
    const int64_t Ntot = T.K * static_cast<int64_t>(T.Np);
    for (size_t p = 0; p < np; ++p)
        if (layout_.gl[p] < 0 || layout_.gl[p] >= Ntot || layout_.gr[p] < 0 || layout_.gr[p] >= Ntot ||
            layout_.stack[p] < 0 || layout_.stack[p] >= static_cast<int32_t>(stacks_.size()))
            throw std::runtime_error("SGBC layout: pair index out of range");
    if (layout_.el_start.size() != layout_.el_elem.size() + 1 || layout_.el_start.back() != static_cast<int32_t>(layout_.ent_face.size()) ||
        layout_.ent_pairs.size() != layout_.ent_face.size() * static_cast<size_t>(T.Nfp))
        throw std::runtime_error("SGBC layout: inconsistent entry tables");
    for (size_t i = 0; i < layout_.el_elem.size(); ++i)
        if (layout_.el_elem[i] < 0 || layout_.el_elem[i] >= T.K || layout_.el_start[i + 1] - layout_.el_start[i] < 1 ||
            layout_.el_start[i + 1] - layout_.el_start[i] > 4)
            throw std::runtime_error("SGBC layout: element entry out of range");
    for (size_t k = 0; k < layout_.ent_face.size(); ++k)
        if (layout_.ent_face[k] < 0 || layout_.ent_face[k] > 3 || layout_.ent_role[k] < 0 || layout_.ent_role[k] > 1)
            throw std::runtime_error("SGBC layout: face entry out of range");
    for (int32_t q : layout_.ent_pairs)
        if (q < 0 || q >= static_cast<int32_t>(np)) throw std::runtime_error("SGBC layout: entry pair out of range");
    try {
        gl_ = upload(layout_.gl); gr_ = upload(layout_.gr); pstack_ = upload(layout_.stack);
        rot_ = upload(layout_.rot); xoff_ = upload(xoff);
        for (int b = 0; b < 2; ++b) {
            X_[b] = zeros<double>(static_cast<size_t>(state_len_));
            snorm_[b] = zeros<double>(np);
        }
        gold_ = zeros<double>(12 * np); gnew_ = zeros<double>(12 * np);
        trace_ = zeros<double>(12 * np); flags_ = zeros<int>(8);
        el_elem_ = upload(layout_.el_elem); el_start_ = upload(layout_.el_start);
        ent_face_ = upload(layout_.ent_face); ent_role_ = upload(layout_.ent_role); ent_pairs_ = upload(layout_.ent_pairs);
        // curved elements' SGBC faces: dense injection blocks, transposed for coalesced reads
        std::vector<char> curved(T.K, 0);
        for (int32_t e : T.curved_elems) curved[e] = 1;
        const int Np = ref.Np, Nfp = ref.Nfp, R = 6 * Np;
        std::vector<int64_t> ent_cblk(layout_.ent_face.size(), -1);
        std::vector<double> cblk, Bm, Bp;
        for (size_t i = 0; i < layout_.el_elem.size(); ++i) {
            const int64_t e = layout_.el_elem[i];
            if (!curved[e]) continue;
            for (int32_t k = layout_.el_start[i]; k < layout_.el_start[i + 1]; ++k) {
                build_curved_sgbc_face(T, ref, alpha, e, layout_.ent_face[k], Bm, Bp);
                ent_cblk[k] = static_cast<int64_t>(cblk.size());
                const size_t o = cblk.size();
                cblk.resize(o + static_cast<size_t>(R) * R + static_cast<size_t>(6 * Nfp) * R);
                for (int r = 0; r < R; ++r)
                    for (int c = 0; c < R; ++c) cblk[o + static_cast<size_t>(c) * R + r] = Bm[static_cast<size_t>(r) * R + c];
                const size_t op = o + static_cast<size_t>(R) * R;
                for (int r = 0; r < R; ++r)
                    for (int c = 0; c < 6 * Nfp; ++c) cblk[op + static_cast<size_t>(c) * R + r] = Bp[static_cast<size_t>(r) * 6 * Nfp + c];
            }
        }
        ent_cblk_ = upload(ent_cblk);
        cblk_ = upload(cblk);
        flux_shmem_ = static_cast<size_t>(std::max(4 * Nfp * 6, 6 * Np + 4 * 6 * Nfp)) * sizeof(double);
    } catch (...) {
        release();
        throw;
    }
}

SgbcOp::~SgbcOp() { release(); }

void SgbcOp::release()
{
    for (auto& kv : maps_) cudaFree(kv.second.a);
    maps_.clear();
    void* bufs[] = {gl_, gr_, pstack_, rot_, xoff_, X_[0], X_[1], snorm_[0], snorm_[1], gold_, gnew_, trace_, flags_,
                    el_elem_, el_start_, ent_face_, ent_role_, ent_pairs_, ent_cblk_, cblk_};
    for (void* b : bufs) if (b) cudaFree(b);
    gl_ = gr_ = pstack_ = nullptr; rot_ = nullptr; xoff_ = nullptr;
    X_[0] = X_[1] = snorm_[0] = snorm_[1] = gold_ = gnew_ = trace_ = nullptr;
    flags_ = nullptr; el_elem_ = el_start_ = ent_face_ = ent_role_ = ent_pairs_ = nullptr;
    ent_cblk_ = nullptr; cblk_ = nullptr;
}

// Called before the maps of one launch are looked up (never between two look-ups of a launch, whose
// pointers go into the same kernel arguments): a Mult at many different times would grow the
// cache without bound, so it starts again once it holds 64 maps (after the device has finished
// with them).
void SgbcOp::trim_maps()
{
    if (maps_.size() + 2 * stacks_.size() <= 64) return;
    ckd(cudaDeviceSynchronize(), "SGBC map cache");
    for (auto& kv : maps_) cudaFree(kv.second.a);
    maps_.clear();
}

const SgbcOp::DevMap& SgbcOp::stage_map(int st, double span, int nsteps)
{
    auto key = std::make_tuple(0, st, span, nsteps);
    auto it = maps_.find(key);
    if (it != maps_.end()) return it->second;
    const SgbcStack1D& S = stacks_[st];
    SgbcStageMap M = sgbc_stage_map(S, span, nsteps);
    std::vector<double> buf(M.R);
    buf.insert(buf.end(), M.G.begin(), M.G.end());
    DevMap d;
    d.a = upload(buf);
    d.n = S.n;
    return maps_.emplace(key, d).first->second;
}

const SgbcOp::DevMap& SgbcOp::final_map(int st, double span, int nsteps)
{
    auto key = std::make_tuple(1, st, span, nsteps);
    auto it = maps_.find(key);
    if (it != maps_.end()) return it->second;
    const SgbcStack1D& S = stacks_[st];
    SgbcFinalMap M = sgbc_final_map(S, span, nsteps);
    std::vector<double> buf(M.FT);
    buf.insert(buf.end(), M.Vo.begin(), M.Vo.end());
    buf.insert(buf.end(), M.Vn.begin(), M.Vn.end());
    DevMap d;
    d.a = upload(buf);
    d.n = S.n;
    return maps_.emplace(key, d).first->second;
}

namespace {

PairArgs pair_args(int64_t np, int64_t N, int32_t* gl, int32_t* gr, int32_t* ps, double* rot, int64_t* xoff,
                   const double* X, const double* snorm, double* Xout, double* snorm_out, double* gold, double* gnew,
                   double* trace, int* flag, const std::vector<SgbcStack1D>& stacks)
{
    PairArgs A{};
    A.n_pairs = np; A.N = N; A.gl = gl; A.gr = gr; A.pstack = ps; A.rot = rot; A.xoff = xoff; A.X = X;
    A.snorm = snorm; A.Xout = Xout; A.snorm_out = snorm_out;
    A.gold = gold; A.gnew = gnew; A.trace = trace; A.flag = flag;
    A.n_stacks = static_cast<int>(stacks.size());
    for (size_t s = 0; s < stacks.size(); ++s) {
        StackInfo& I = A.st[s];
        I.n = stacks[s].n; I.local = stacks[s].local; I.idx_left = stacks[s].idx_left; I.idx_right = stacks[s].idx_right;
        I.left_bc = stacks[s].spec.left_bc; I.right_bc = stacks[s].spec.right_bc;
    }
    return A;
}

}  // namespace

void SgbcOp::commit(const TablesDev& T, const double* x, double t, double dt, cudaStream_t s)
{
    cp_ = cur_;
    base_ = t;
    step_dt_ = dt;
    // the ghost values of the step's start state (the trace kernel without an advance)
    PairArgs P = pair_args(n_pairs(), T.N, gl_, gr_, pstack_, rot_, xoff_, X_[cp_], snorm_[cp_], nullptr, nullptr,
                           gold_, gnew_, trace_, flags_ + 6, stacks_);
    ckd(cudaMemsetAsync(flags_ + 6, 0, sizeof(int), s), "SGBC flag reset");
    const int grid = static_cast<int>(std::min<int64_t>(kGridCap, (n_pairs() + 7) / 8));
    sgbc_trace_kernel<<<std::max(1, grid), 256, 0, s>>>(P, x, 0, 1);
    ckd(cudaGetLastError(), "SGBC trace kernel");
    ++launches_;
}

void SgbcOp::before_stage(const TablesDev& T, const StageArgs& A, double t, cudaStream_t s)
{
    if (A.batch != 1) throw std::invalid_argument("thin-layer (SGBC) sub-solvers need a single incidence");
    double span = 0.0, nominal = 0.0;
    int store_old = 0;
    switch (A.mode) {
    case MODE_MULT: {
        // a Mult at stage time t: (t + c dt) - t differs from c dt by rounding only, so a cached
        // map of a span within a few ulps of t is reused rather than rebuilt every step
        span = t - base_;
        nominal = span;
        const double tol = 8.0 * std::numeric_limits<double>::epsilon() * std::max(1.0, std::fabs(t));
        for (const auto& kv : maps_) {
            const auto& k = kv.first;
            if (std::get<0>(k) == 0 && std::fabs(std::get<2>(k) - span) <= tol) { nominal = std::get<2>(k); break; }
        }
        break;
    }
    case MODE_RK4_1:   // the step's checkpoint (Solver::step, Solver.cpp:535-542)
        cp_ = cur_; base_ = t; step_dt_ = A.dt; span = 0.0; store_old = 1;
        break;
    case MODE_RK4_2:
    case MODE_RK4_3: span = t - base_; nominal = 0.5 * A.dt; break;
    case MODE_RK4_4: span = t - base_; nominal = A.dt; break;
    default:
        throw std::invalid_argument("thin-layer (SGBC) sub-solvers are coupled to classical RK4 (DGTD_RK4) and Mult");
    }
    const int advance = span > 1e-12 ? 1 : 0;
    cur_flag_ = (A.mode == MODE_MULT) ? 0 : A.mode;
    if (advance) trim_maps();
    PairArgs P = pair_args(n_pairs(), T.N, gl_, gr_, pstack_, rot_, xoff_, X_[cp_], snorm_[cp_], nullptr, nullptr,
                           gold_, gnew_, trace_, flags_ + cur_flag_, stacks_);
    if (advance)
        for (int st = 0; st < n_stacks(); ++st) {
            const DevMap& M = stage_map(st, nominal, sgbc_nsteps(stacks_[st].spec.sub_dt, span));
            P.st[st].R = M.a;
            P.st[st].G = M.a + 12 * M.n;
        }
    ckd(cudaMemsetAsync(flags_ + cur_flag_, 0, sizeof(int), s), "SGBC flag reset");
    const int grid = static_cast<int>(std::min<int64_t>(kGridCap, (n_pairs() + 7) / 8));
    sgbc_trace_kernel<<<std::max(1, grid), 256, 0, s>>>(P, A.in, advance, store_old);
    ckd(cudaGetLastError(), "SGBC trace kernel");
    ++launches_;
}

void SgbcOp::after_stage(const TablesDev& T, const StageArgs& A, cudaStream_t s)
{
    FluxArgs F{};
    F.in = A.in; F.trace = trace_; F.flag = flags_ + cur_flag_;
    F.n_elems = static_cast<int64_t>(layout_.el_elem.size());
    F.el_elem = el_elem_; F.el_start = el_start_; F.ent_face = ent_face_; F.ent_role = ent_role_; F.ent_pairs = ent_pairs_;
    F.ent_cblk = ent_cblk_; F.cblk = cblk_;
    F.mode = A.mode; F.dt = A.dt; F.out = A.out; F.yout = A.yout; F.z = A.z; F.x = A.x;
    const size_t shmem = flux_shmem_;
    const int grid = static_cast<int>(std::min<int64_t>(kGridCap, std::max<int64_t>(1, F.n_elems)));
    sgbc_flux_kernel<<<grid, 128, shmem, s>>>(T, F);
    ckd(cudaGetLastError(), "SGBC flux kernel");
    ++launches_;
    if (A.mode == MODE_RK4_4) finalize(T, A.x, s);
}

void SgbcOp::finalize(const TablesDev& T, const double* x, cudaStream_t s)
{
    const int out = 1 - cp_;
    trim_maps();
    PairArgs P = pair_args(n_pairs(), T.N, gl_, gr_, pstack_, rot_, xoff_, X_[cp_], snorm_[cp_], X_[out], snorm_[out],
                           gold_, gnew_, trace_, flags_ + 7, stacks_);
    int64_t n_max = 0;
    for (int st = 0; st < n_stacks(); ++st) {
        const DevMap& M = final_map(st, step_dt_, sgbc_nsteps(stacks_[st].spec.sub_dt, step_dt_));
        P.st[st].FT = M.a;
        P.st[st].Vo = M.a + M.n * M.n;
        P.st[st].Vn = M.a + M.n * M.n + 12 * M.n;
        n_max = std::max(n_max, M.n);
    }
    ckd(cudaMemsetAsync(flags_ + 7, 0, sizeof(int), s), "SGBC flag reset");
    const int qgrid = static_cast<int>(std::max<int64_t>(1, (n_pairs() + 255) / 256));
    sgbc_quiesce_kernel<<<qgrid, 256, 0, s>>>(P, x);
    ckd(cudaGetLastError(), "SGBC quiescence kernel");
    const size_t fsh = static_cast<size_t>(n_max + 24) * sizeof(double);
    const int fgrid = static_cast<int>(std::min<int64_t>(kGridCap, std::max<int64_t>(1, n_pairs())));
    sgbc_final_kernel<<<fgrid, 256, fsh, s>>>(P, n_max);
    ckd(cudaGetLastError(), "SGBC final kernel");
    launches_ += 2;
    cur_ = out;
}

void SgbcOp::read_states(double* host) const
{
    ckd(cudaMemcpy(host, X_[cur_], static_cast<size_t>(state_len_) * sizeof(double), cudaMemcpyDeviceToHost),
        "cudaMemcpy SGBC states");
}

}  // namespace dgtd
