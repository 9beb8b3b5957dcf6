/*
 * dgtd_gb300 — C ABI of the GB300-native DG time-domain Maxwell step.
 *
 * This is the boundary that replaces the reference's evolution operator
 * (class maxwell::GlobalEvolution : mfem::TimeDependentOperator,
 * src/evolution/GlobalEvolution.h:14-111) and the time loop that drives it
 * (maxwell::Solver::run/step, src/solver/Solver.cpp:483-551).
 *
 * Conventions
 *  - Every call returns DGTD_OK (0) or a negative error code; no exception
 *    crosses the ABI. dgtd_last_error() returns a thread-local message.
 *  - State vectors use the reference layout (src/evolution/Fields.h:48-65):
 *    [Ex | Ey | Ez | Hx | Hy | Hz], each block K*Np doubles, element-major,
 *    nodes in the order of L2_FECollection(p, 3, GaussLobatto). A batched
 *    operator (batch B > 1) stacks B such vectors back to back.
 *  - Pointers named d_* are device pointers; h_* are host pointers.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).
 *  - One operator per stream at a time: calls on one operator are not
 *    re-entrant (the reference's Mult mutates work vectors, GlobalEvolution.h:82-110).
 */
#ifndef DGTD_GB300_H
#define DGTD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DGTD_OK 0
#define DGTD_ERR_INVALID (-1)
#define DGTD_ERR_CUDA (-2)
#define DGTD_ERR_UNSUPPORTED (-3)
#define DGTD_ERR_NOMEM (-4)
#define DGTD_ERR_TIMEOUT (-5)
#define DGTD_ERR_UNSTABLE (-6) /* the run loop's instability detector tripped (stop mode) */

/* Boundary codes (reference BdrCond, src/components/Types.h:47-55). */
#define DGTD_BC_OPEN 0
#define DGTD_BC_PEC 1
#define DGTD_BC_PMC 2
#define DGTD_BC_SMA 3
#define DGTD_BC_SGBC 4   /* interior faces only: a thin-layer stack (dgtd_op_set_sgbc) */

/* Precision forms. */
#define DGTD_FP64 0        /* plain form: FP64 state and arithmetic */
#define DGTD_FP32_3XTF32 1 /* batched form: FP32 state, 3xTF32 tensor-core contractions */
#define DGTD_FP32 2        /* single-instance form: FP32 state in the reference layout, FP32 arithmetic */

/* Time integrators. */
#define DGTD_RK4 0    /* classical RK4, mfem::RK4Solver semantics (reference default, Solver.cpp:45-47) */
#define DGTD_LSERK4 1 /* 5-stage low-storage RK4 (Carpenter & Kennedy 1994) */

/*
 * Mesh description (replaces the MFEM ParMesh + Model of the reference:
 * element attributes -> per-element eps/mu/sigma, Model.cpp:145-161;
 * boundary attributes -> codes, driver.cpp:870-887; TF/SF interior faces,
 * SubMesher.cpp:359-775).
 */
typedef struct dgtd_mesh_desc {
    int32_t dim;                /* 3 (tetrahedra) */
    int64_t n_vertices;
    const double* vertices;     /* [n_vertices][3] */
    int64_t n_elements;
    const int32_t* elements;    /* [n_elements][4], positively oriented */
    const double* eps_r;        /* [n_elements] or NULL (1) */
    const double* mu_r;         /* [n_elements] or NULL (1) */
    const double* sigma;        /* [n_elements] or NULL (0) */
    int64_t n_bdr_faces;
    const int32_t* bdr_faces;   /* [n_bdr_faces][3] vertex ids */
    const int32_t* bdr_codes;   /* [n_bdr_faces] DGTD_BC_* */
    int64_t n_tfsf_faces;
    const int32_t* tfsf_faces;  /* [n][3], winding normal points into the total-field side */
    int64_t n_int_faces;
    const int32_t* int_faces;   /* [n][3] interior PEC/PMC/SMA sheets */
    const int32_t* int_codes;   /* [n] DGTD_BC_PEC/PMC/SMA/SGBC */
    /* second-order (curved) elements: their ids and geometry nodes [n_curved][10][3] = the
     * element's four corners (its vertex order) then the nodes on its edges (0,1) (0,2) (0,3)
     * (1,2) (1,3) (2,3). They are assembled on their isoparametric map (FP64 form only; no TF/SF
     * faces on them). n_curved = 0 for affine meshes. */
    int64_t n_curved;
    const int32_t* curved_elems;
    const double* curved_nodes;
} dgtd_mesh_desc;

typedef struct dgtd_op_opts {
    int32_t order;      /* polynomial order p, 1..6 (reference solver_options.order) */
    double alpha;       /* upwind coefficient (reference solver_options.upwind_alpha) */
    int32_t precision;  /* DGTD_FP64, DGTD_FP32_3XTF32 or DGTD_FP32 */
    int32_t batch;      /* B incidences sharing the mesh (>= 1) */
} dgtd_op_opts;

/* Gaussian / modulated-Gaussian plane wave (reference Planewave, Function.h:329-416,
 * built by driver.cpp:483-519; mean is the 1D Gaussian mean along the propagation). */
typedef struct dgtd_planewave {
    double propagation[3]; /* normalised by the library */
    double polarization[3];/* normalised by the library */
    double spread;
    double mean;
    double frequency;      /* 0: plain Gaussian; else carrier (normalised units) */
    int32_t batch;         /* incidence index in [0, B) */
} dgtd_planewave;

typedef struct dgtd_op_info {
    int64_t n_elements;
    int32_t order, np, nfp;
    int32_t batch;
    int32_t precision;
    int64_t ndofs;          /* K*Np (per field component) */
    int64_t state_len;      /* 6*K*Np*B entries of the reference-layout state */
    int64_t n_tfsf_faces;   /* element faces flagged TF/SF (counted per side) */
    double min_edge;
    double dt_scale_min;    /* min over elements of vol / (sum of face areas / 2) */
    int64_t device_bytes;   /* bytes of device tables held by the operator */
    int64_t work_len;       /* entries of the operator's working state (dgtd_op_step / dgtd_op_mult):
                               FP64 form: = state_len (reference layout);
                               batched FP32 form: 2*K*6*Np*Bpad floats: the x_hi block then the x_lo
                               block (each element-blocked, incidence fastest; classical RK4 keeps the
                               state as that FP32 pair, the other forms and stage inputs read x_hi);
                               single-instance FP32 form: = state_len floats (reference layout) */
    int32_t work_word_bytes;/* 8 (FP64 form) or 4 (FP32 forms) */
    int32_t batch_padded;   /* B rounded up to the incidence chunk (FP32 form), else B */
} dgtd_op_info;

typedef struct dgtd_op dgtd_op;

/* Thread-local description of the last error. */
const char* dgtd_last_error(void);

/* Number of CUDA kernels this library has launched in the process so far. */
uint64_t dgtd_kernel_launches(void);

/* Operator life cycle (reference GlobalEvolution ctor, GlobalEvolution.cpp:32-364:
 * here the once-per-mesh work is the geometric-factor / LIFT / node-map build). */
int dgtd_op_create(const dgtd_mesh_desc* mesh, const dgtd_op_opts* opts, dgtd_op** out);
void dgtd_op_destroy(dgtd_op* op);
int dgtd_op_get_info(const dgtd_op* op, dgtd_op_info* info);

/* Physical coordinates of every DOF node: h_xyz is [3][K*Np]
 * (reference buildDoFPositions, HesthavenEvolutionMethods.cpp:77-91). */
int dgtd_op_node_coords(const dgtd_op* op, double* h_xyz);

/* Replace the plane-wave sources (reference TotalField sources handled by
 * GlobalEvolution::applyTFSFSourceToVector, GlobalEvolution.cpp:551-626). */
int dgtd_op_set_planewaves(dgtd_op* op, const dgtd_planewave* pw, int32_t n);

/* y = dU/dt(x, t): exact TimeDependentOperator::Mult semantics
 * (reference GlobalEvolution::Mult, GlobalEvolution.cpp:628-1088).
 * d_x, d_y: device working states (work_len entries of work_word_bytes each;
 * the reference layout for the FP64 form), must not alias. */
int dgtd_op_mult(dgtd_op* op, const void* d_x, void* d_y, double t, void* stream);

/* Convert between the reference layout (FP64, [b][c][e*Np+i]) and the operator's working
 * state (device). Identity copy for the FP64 form. d_ref may be device memory or pinned
 * (page-locked) host memory: the conversion kernel then reads or writes the host buffer over
 * the host link, fusing the transfer with the conversion. Pageable host memory is rejected
 * with DGTD_ERR_INVALID. The batched form's working state holds each value as an FP32 pair
 * (x_hi = fl(x), x_lo = fl(x - x_hi)), so pack/unpack keep about 48 bits of the FP64 value. */
int dgtd_op_pack(dgtd_op* op, const double* d_ref, void* d_work, void* stream);
int dgtd_op_unpack(dgtd_op* op, const void* d_work, double* d_ref, void* stream);

/* Same as dgtd_op_mult with host buffers: copies in, applies, copies out
 * (synchronous). */
int dgtd_op_mult_host(dgtd_op* op, const double* h_x, double* h_y, double t);

/* Advance d_state (device working state) by nsteps steps of size dt from t0
 * with the fused stage kernels (reference Solver::step + mfem RK4Solver::Step,
 * Solver.cpp:535-551). The operator keeps its RK registers in device scratch it
 * allocates on first use. */
int dgtd_op_step(dgtd_op* op, void* d_state, double t0, double dt, int32_t nsteps, int32_t integrator,
                 void* stream);

/* Run to final_time from t0 following the reference loop (Solver::run,
 * Solver.cpp:483-551: while t <= T - 1e-8 dt, last step truncated to T - t).
 * h_state: host, in/out. Returns the number of steps taken in *steps_out. */
int dgtd_op_run_host(dgtd_op* op, double* h_state, double t0, double dt, double final_time, int32_t integrator,
                     int64_t* steps_out);

/* Same as dgtd_op_step on the FP64 form, but allocating nothing: the three RK
 * registers live in one fixed file-scope device array of 3 * dgtd_noalloc_max_state()
 * doubles (24 MiB), shared by all operators and calls in the process. No counterpart
 * in the reference; it serves callers that cannot allow a device allocation during
 * stepping. The first call on each device looks up the array's address (set-up: make
 * that call before any stream capture). Errors: DGTD_ERR_INVALID when state_len
 * exceeds dgtd_noalloc_max_state(), DGTD_ERR_UNSUPPORTED for the FP32 forms and for
 * meshes with thin-layer (SGBC) faces (their sub-step maps are built on first use).
 * Installed probes (dgtd_op_set_probes) are sampled after every `every`-th step on the
 * same step counter as dgtd_op_step, so the two calls may be mixed on one operator.
 * The array keeps the last call's contents; calls that overlap on the GPU race. */
int dgtd_op_step_noalloc(dgtd_op* op, void* d_state, double t0, double dt, int32_t nsteps, int32_t integrator,
                         void* stream);

/* Instability detector of dgtd_op_run_host (reference Solver::run, Solver.cpp:500-516,
 * which checks the field norm after every step and prints a warning when it is not finite
 * or above 1e20). Here a device reduction runs every `every` steps (default 10; 0 turns it
 * off) and after the last step, without host synchronisation; the host reads the result
 * every 256 steps and at the end. stop = 0 (default) follows the reference: a warning on
 * stderr and the run goes on; stop = 1 ends the run at the next read with
 * DGTD_ERR_UNSTABLE. */
int dgtd_op_set_stability_check(dgtd_op* op, int32_t every, int32_t stop);

/* The detector's record (of the last dgtd_op_run_host, or of the checks since the last
 * dgtd_op_stability_reset): the step count and time of the first check that tripped
 * (first_step = -1: none), its norm, and the number of checks run. Outputs may be NULL. */
int dgtd_op_stability(const dgtd_op* op, int64_t* first_step, double* t, double* norm, int64_t* checks);

/* For callers that run their own loop (the adapter under Solver::run): one check of the
 * working state d_state at step count `step` and time t on `stream` (device reduction, no
 * host synchronisation; the record keeps the first check that tripped), and a reset of the
 * record. */
int dgtd_op_stability_check(dgtd_op* op, const void* d_state, int64_t step, double t, void* stream);
int dgtd_op_stability_reset(dgtd_op* op);

/* Largest state_len (reference-layout entries) dgtd_op_step_noalloc accepts. */
int64_t dgtd_noalloc_max_state(void);

/* Contraction path of the FP32 forms: 0 = tensor cores (tcgen05, 3xTF32) where supported,
 * else FP32 SIMT; 1 = FP32 SIMT. Batched form (default 0): tensor cores for orders 1..4 with
 * B padded to a multiple of 64 (work item: one element x 64 incidences). Single-instance
 * form (default 1: its SIMT stage takes 0.91 x the tensor-core stage's time at p = 6 on
 * GB300): tensor cores for orders 1..6 (work item: 8 elements of one incidence; reference-
 * element matrices as the A operand, fields and fluxes as the B operand, chain rule and curl
 * in FP32 in the epilogue). */
int dgtd_op_set_contraction(dgtd_op* op, int32_t mode);

/* Batched FP32 form: replay blocks of `steps` classical-RK4 steps of dgtd_op_step from one
 * captured CUDA graph (stage times read from a device scalar the graph advances); 0 turns
 * it off (default). Used only on a non-default stream (the legacy stream cannot be
 * captured) and without probes; the first call with a new state pointer, dt or stream
 * captures the graph. DGTD_ERR_UNSUPPORTED for the other forms. */
int dgtd_op_set_graph_steps(dgtd_op* op, int32_t steps);

/* Batched FP32 form, classical RK4: FP64 defect correction of the operator (no counterpart in
 * the reference, whose operator is FP64 throughout). Every `every` steps of dgtd_op_step (0: off,
 * the default) the state is unpacked, the plain FP64 form applies the operator to it, and the
 * difference c = L64(x) - L32(x_hi) from this form's product of the same state is formed (bf16,
 * one state block). c is kept where the state has stayed within 0.1 of the incidence's RMS value
 * of its value at the previous refresh: there the field stays put (a static remainder, a slowly
 * varying mode; the scale is per incidence because a static field's drift builds up in components
 * near zero, such as H beside a static E) and
 * its FP32 rounding would otherwise repeat step after step and accumulate into a drift; where the
 * field moves, its rounding error is random from step to step and a stale c held for a whole
 * refresh period would make it systematic, so c is left out. The first refresh of a trajectory
 * therefore applies nothing. The operator is linear, so adding c to every stage's right-hand side
 * adds, per step, the increment dt (1 + dtL/2 + (dtL)^2/6 + (dtL)^3/24) c: it is formed once per
 * refresh and dt (three source-free FP32 products) and added to the state's low word after every
 * step by an elementwise kernel; the stage kernels are unchanged.
 * The correction belongs to the trajectory being stepped: it is also refreshed at the first step
 * after this call, when dgtd_op_step is given another state buffer, after
 * dgtd_op_set_planewaves and at the start of dgtd_op_run_host (these also forget the previous
 * state), but not by dgtd_op_pack (a caller that moves the state through the reference layout
 * every step keeps it). A caller that loads an unrelated state into the same buffer calls this
 * function again; until then a stale correction adds a forcing at the FP32 rounding level of the
 * old state's right-hand side. Costs per refresh: unpack, one FP64 product, pack and four FP32
 * products; per step one elementwise pass (read x_lo and the bf16 increment, write x_lo); in
 * device memory two scratch buffers of max(FP64 reference state, FP32 working state) bytes, one
 * FP32 state block and two bf16 blocks. Steps run one at a time (no CUDA-graph replay). Mult does
 * not add the correction. DGTD_ERR_UNSUPPORTED for the other forms, and from dgtd_op_step with
 * DGTD_LSERK4 while the correction is on. */
int dgtd_op_set_defect_correction(dgtd_op* op, int32_t every);

/* Refreshes made by the defect correction since the operator was created (may be NULL). */
int dgtd_op_defect_refreshes(const dgtd_op* op, int64_t* refreshes);

/* Batched FP32 form: time the candidate stage kernels on this operator's mesh and keep the
 * fastest (the tile-shape autotuner): 0 = tensor cores (3xTF32, 64 incidences x one element
 * per work item; orders 1..4, B padded to 64), 1..3 = FP32 SIMT with 4, 8, 16 warps per
 * block (32 incidences x one element per block). d_work: a working state (device; read
 * only). h_ms[4] (may be NULL) gets each candidate's mean launch time in ms (-1: not
 * applicable); *choice gets the index kept. Results are cached per (order, padded batch,
 * element count) for the process. DGTD_ERR_UNSUPPORTED for the other forms. */
int dgtd_op_autotune(dgtd_op* op, const void* d_work, void* stream, double* h_ms, int32_t* choice);

/* 1 when an FP32 form (batched or single-instance) runs its contractions on the tensor cores
 * with the current contraction setting, else 0. */
int dgtd_op_uses_tensor_cores(const dgtd_op* op);

/* Synchronise the stream and report device-side failures of earlier calls
 * (a bounded wait inside a kernel that gave up): DGTD_OK or DGTD_ERR_TIMEOUT. */
int dgtd_op_check(dgtd_op* op, void* stream);

/* Squared L2 norm per incidence: h_out[b] (host, B entries) of a working state (device). */
int dgtd_op_norm2(dgtd_op* op, const void* d_state, double* h_out, void* stream);

/* Automatic time step of the reference's 3D Global operator
 * (estimateTimeStep, Solver.cpp:289-300, 349-351) at the given cfl. */
int dgtd_op_estimate_dt(const dgtd_op* op, double cfl, double* dt_out);

/* ---- probes: point probes and running FP64 DFT accumulators ---------------------
 *
 * Replace the reference's point probes (PointProbe, src/components/Probes.h:132-160;
 * ProbesManager::updateProbe, src/solver/ProbesManager.cpp:380-405) and the DFT of
 * exported surface snapshots done by the near-to-far post-processor
 * (RCSSurfacePostProcessor.cpp:274-300). Sums are accumulated on the device in
 * FP64 after every `every`-th step of dgtd_op_step, or by dgtd_op_probe_sample:
 *   S(f) = sum_n u(t_n) exp(-i 2 pi f t_n)      (the reference divides by the sample count)
 * for every field component of every point probe and surface node. */
typedef struct dgtd_probe_spec {
    int32_t n_points;
    const double* points;          /* [n_points][3]; each must lie in the mesh */
    int64_t n_surface_faces;
    const int32_t* surface_faces;  /* [n][3] vertex ids of mesh faces (near-to-far surface);
                                      winding normal points out of the enclosed region */
    int32_t n_freqs;               /* 0..64 */
    const double* freqs;           /* cycles per unit time */
    int32_t every;                 /* dgtd_op_step samples after every `every`-th step (>= 1) */
    int32_t max_records;           /* point time-series capacity in samples (0: no series) */
} dgtd_probe_spec;

/* Install probes (replaces earlier ones; sums start at zero; the step counter restarts). */
int dgtd_op_set_probes(dgtd_op* op, const dgtd_probe_spec* spec);

/* ---- thin-layer boundaries (SGBC) ----------------------------------------------------------
 * A stack of thin layers on interior faces, each face node pair coupled to its own 1D DG
 * sub-solver (reference SGBCWrapper, src/solver/SolverExtension.cpp:49-559, and its coupling in
 * GlobalEvolution, src/evolution/GlobalEvolution.cpp:48-300, 395-545, 639-1001):
 *  - the sub-solver mesh is the layers with max(3, p+1) vacuum ghost segments on each side
 *    (width = total width / total segments), SMA at its two ends, and the stack's optional
 *    sheets at the ghost/layer interfaces; order p = max over layers; upwind alpha 1; SDIRK33
 *    steps with a dense implicit solve (at most 600 sub-solver unknowns: larger stacks fail with
 *    DGTD_ERR_UNSUPPORTED, the reference iterates with GMRES there);
 *  - the pair of a face node is (node of the face's first element = the lower element index,
 *    partner node of the second); the sub-solver's x axis is the first element's outward normal,
 *    its left ghosts hold the first node's fields and its right ghosts the second's;
 *  - every RK stage restarts the sub-solvers from the step's start and advances them to the stage
 *    time (ceil(span / sub_dt) sub-steps) with the stage input as ghost data; the face flux of
 *    the first element then takes the slab's left interface value as neighbour trace (or the left
 *    sheet's mirror of its own value), the second element the right one; after the step the
 *    sub-solvers advance over the whole step with ghosts interpolated between its two ends;
 *  - pairs, and the whole coupling, are skipped while their fields stay below 1e-8.
 * The FP64 form with one incidence and classical RK4 (and dgtd_op_mult) only:
 * DGTD_ERR_UNSUPPORTED for the other forms, batches, LSERK4 and dgtd_op_step_noalloc. Before
 * dgtd_op_set_sgbc, stepping an operator whose mesh has DGTD_BC_SGBC faces fails with
 * DGTD_ERR_UNSUPPORTED. dgtd_op_mult at time t advances the checkpoint (the states at the last
 * step's start; zero, at time 0, before the first) over t minus that start. */
typedef struct dgtd_sgbc_layer {
    double eps_r, mu_r;
    double sigma;        /* conductivity in solver units (S/m times the free-space impedance) */
    double width;        /* mesh units */
    int32_t segments;    /* sub-solver segments across the layer (>= 1) */
    int32_t order;       /* polynomial order (1..16; the stack uses the largest) */
} dgtd_sgbc_layer;

typedef struct dgtd_sgbc_stack {
    int32_t n_layers;
    const dgtd_sgbc_layer* layers;   /* first layer next to the faces' first elements */
    int32_t left_bc, right_bc;       /* 0: none, or DGTD_BC_PEC/PMC/SMA sheet on that side */
    double sub_dt;                   /* the sub-solver's step (normalised time), the reference's
                                        SGBCWrapper::getRecommendedDt; <= 0: one sub-step per span */
} dgtd_sgbc_stack;

/* face_stack[i]: stack of the i-th interior face given with DGTD_BC_SGBC (mesh order). The
 * sub-solver states start at zero. */
int dgtd_op_set_sgbc(dgtd_op* op, const dgtd_sgbc_stack* stacks, int32_t n_stacks, const int32_t* face_stack);
/* The step hooks of the reference's Solver::step (Solver.cpp:535-551) for callers that drive
 * their own integrator with dgtd_op_mult: commit before the step's first stage (the states become
 * the checkpoint every Mult restarts from; t the step's start, dt its length, d_x its start
 * state; GlobalEvolution::commitSGBCCheckpoint) and finalize after its last (the states advance
 * from the checkpoint over dt with ghosts interpolated towards d_x, the step's end state;
 * GlobalEvolution::finalizeSGBCStep). dgtd_op_step does both itself. */
int dgtd_op_sgbc_commit(dgtd_op* op, const void* d_x, double t, double dt, void* stream);
int dgtd_op_sgbc_finalize(dgtd_op* op, const void* d_x, void* stream);
/* Pairs and total sub-solver unknowns (0, 0 without SGBC); h_states (if not NULL, capacity
 * `cap` entries) receives the pairs' states, pair after pair. */
int dgtd_op_sgbc_states(const dgtd_op* op, int64_t* n_pairs, int64_t* state_len, double* h_states, int64_t cap);

/* Node sets of the order-p tetrahedron (no GPU). The operator's state holds nodal values on MFEM's
 * Gauss-Lobatto L2 node set; the reference's solver_options.basis_type 0 selects MFEM's
 * Gauss-Legendre set of the same polynomial space (L2_FECollection(p, 3, BasisType::GaussLegendre),
 * Solver.cpp:86). The reference's integration rules are exact on straight elements (faces: order
 * 2p + 1, IntegratorFunctions.cpp:7-35; volume: 2p - 1 and 2p), so its operator in either basis is
 * the same semi-discrete system: A_legendre = M(lobatto -> legendre) A M(legendre -> lobatto),
 * element by element. */
#define DGTD_BASIS_GAUSS_LEGENDRE 0
#define DGTD_BASIS_GAUSS_LOBATTO 1
/* Barycentric coordinates [Np][4] (l0..l3, on the element's vertices 0..3) of the nodes of a
 * basis type, in DOF order. */
int dgtd_tet_nodes(int32_t order, int32_t basis_type, double* bary);
/* [Np][Np] row-major M with v_to = M v_from for the nodal values of any degree-p polynomial. */
int dgtd_tet_basis_change(int32_t order, int32_t from_basis, int32_t to_basis, double* m);
/* The same change applied on the device to a whole FP64 reference-layout state (state_len
 * values; d_in and d_out distinct): a Gauss-Legendre caller runs
 * change(GL -> GLL), dgtd_op_mult / dgtd_op_step, change(GLL -> GL). One kernel launch. */
int dgtd_op_change_basis(dgtd_op* op, const void* d_in, void* d_out, int32_t from_basis, int32_t to_basis,
                         void* stream);

/* Host-side rows of the curved elements of a mesh (no GPU): elems [n_curved], nbr [n_curved][4]
 * (face neighbour or -1) and blocks [n_curved][5][6 Np][6 Np] (row-major; rows (component, node)
 * of dU/dt, columns (component, node) of the element's own state, block 0, or of its neighbour
 * across face f, block 1 + f). cap = entries available in blocks. */
int dgtd_curved_block_rows(const dgtd_mesh_desc* mesh, int32_t order, double alpha, int32_t* elems, int32_t* nbr,
                           double* blocks, int64_t cap);

/* Host-side tables of one stack (no GPU): the sub-solver's size n and operator A [n][n]
 * (A may be NULL to query n; cap = entries available in A), and its interface rows. */
int dgtd_sgbc_stack_operator(const dgtd_sgbc_stack* stack, int64_t* n, int64_t* idx_left, int64_t* idx_right,
                             double* A, int64_t cap);
/* The composed maps of nsteps sub-steps over span (no GPU): with ghosts held at g, the 12
 * interface values (left E,H then right E,H, face frame) are R x + G g, R [12][n], G [12][12];
 * with ghosts interpolated from g_old to g_new, the state is F x + Vo g_old + Vn g_new, F [n][n],
 * Vo and Vn [n][12]. Any output may be NULL. */
int dgtd_sgbc_stack_maps(const dgtd_sgbc_stack* stack, double span, int32_t nsteps, double* R, double* G, double* F,
                         double* Vo, double* Vn);
int dgtd_op_clear_probes(dgtd_op* op);
/* Zero the sums and the time series. */
int dgtd_op_probe_reset(dgtd_op* op, void* stream);
int dgtd_op_probe_info(const dgtd_op* op, int64_t* n_surface_nodes, int64_t* n_samples, int64_t* n_records);
/* Surface nodes: coordinates [n][3], unit outward normals [n][3], quadrature weights [n]
 * (sum of the weights = surface area). Any pointer may be NULL. */
int dgtd_op_probe_surface(const dgtd_op* op, double* h_xyz, double* h_normal, double* h_weight);
/* Add one sample of a working state (device) at time t. */
int dgtd_op_probe_sample(dgtd_op* op, const void* d_state, double t, void* stream);
/* Read (synchronising `stream`): point sums [B][n_points][6][n_freqs][2] (re, im),
 * surface sums [B][n_surface_nodes][6][n_freqs][2], point series [n_records][B][n_points][6]
 * and its times [n_records]. Any pointer may be NULL. */
int dgtd_op_probe_read(dgtd_op* op, double* h_point_dft, double* h_surface_dft, double* h_series, double* h_series_t,
                       void* stream);

/* ---- JSON cases --------------------------------------------------------------
 *
 * The reference's case files (driver::buildSolverJson, src/driver/driver.cpp:1545:
 * solver_options, model {filename (gmsh 2.2 ASCII), refinement, materials,
 * boundaries}, sources {initial, planewave}, probes {point, rcssurface, farfield})
 * loaded into this library's tables, with SGBC layers (dgtd_case_sgbc) and curved second-order
 * tetrahedra (their geometry in dgtd_case_mesh; refinement keeps children on the parent's map).
 * Unsupported features (dipoles, 1D/2D meshes, TF/SF faces on curved elements) are rejected
 * with an error. */
typedef struct dgtd_case dgtd_case;

typedef struct dgtd_case_info {
    int32_t order;
    int32_t integrator;          /* DGTD_RK4 / DGTD_LSERK4 (solver_options.ode_type) */
    double alpha;
    double time_step;            /* 0: estimated from cfl */
    double final_time;
    double cfl;
    int32_t n_waves;
    int32_t n_initial_fields;
    int32_t n_point_probes;
    int32_t n_surfaces;
    int64_t n_elements;
    int64_t n_vertices;
    int32_t n_sgbc_stacks;       /* "SGBC" boundary entries (dgtd_case_sgbc) */
    int32_t n_sgbc_layers;       /* layers over all stacks */
    int64_t n_sgbc_faces;        /* interior faces given with DGTD_BC_SGBC in the case mesh */
    int32_t basis_type;          /* solver_options.basis_type: DGTD_BASIS_GAUSS_LOBATTO (default) or
                                    DGTD_BASIS_GAUSS_LEGENDRE; dgtd_case_run then takes the initial
                                    fields at the Gauss-Legendre nodes and returns the final state
                                    on them (the operator runs on the Gauss-Lobatto set between) */
} dgtd_case_info;

typedef struct dgtd_case_run_opts {
    int32_t precision;           /* DGTD_FP64 (the plain form) */
    const double* freqs;         /* DFT frequencies of the point probes and surfaces (may be NULL) */
    int32_t n_freqs;
    const char* out_dir;         /* if not NULL: PointProbe<k>.dat files in the reference's layout
                                    (ProbesManager.cpp:203-215, 400-407): four header lines, then
                                    t Ex Ey Ez Hx Hy Hz per sample with t in seconds (t / c) */
} dgtd_case_run_opts;

typedef struct dgtd_case_result {
    int64_t steps;
    double dt;
    double final_time;
    int64_t n_records;           /* point-probe samples recorded */
    double seconds;              /* wall time of the time loop */
    int64_t unstable_step;       /* first step whose field norm was not finite or above 1e20, checked
                                    every 10 steps and at the end (reference Solver.cpp:500-516; the
                                    run goes on after a warning on stderr, as the reference's), or -1 */
} dgtd_case_result;

/* Read a case file and its mesh (reference driver::buildSolverJson, driver.cpp:1545, with its
 * case layout, driver.cpp:1487-1543: <case>/<case>.json beside <case>/<case>.msh, and
 * model.filename = "<case>.msh"; other layouts fail with DGTD_ERR_INVALID and a message naming
 * what differs). */
int dgtd_case_load(const char* json_path, dgtd_case** out);
void dgtd_case_destroy(dgtd_case* c);
int dgtd_case_get_info(const dgtd_case* c, dgtd_case_info* info);
/* The case's thin-layer stacks (n_sgbc_stacks entries; their `layers` point into `layers`,
 * n_sgbc_layers entries) and the stack of each DGTD_BC_SGBC face (n_sgbc_faces), ready for
 * dgtd_op_set_sgbc. A "SGBC" boundary entry (driver.cpp:1298-1462) takes "material" (one layer) or
 * "layers"; a layer needs "bulk_conductivity" (S/m) and "material_width", takes
 * "relative_permittivity" / "relative_permeability" (1), and an automatic order (2, 3 or 4 by
 * its loss tangent at the pulses' top frequency) and segment count (20 nodes per wavelength and
 * two segments per skin depth, 4..1000) unless "order" / "num_of_segments" are given;
 * "sgbc_boundaries": {"left", "right"} (PEC/PMC/SMA) at the entry or, when absent there, in its
 * material. The sub-step is half a segment's wave crossing time, relaxed by min(N^2, 50) for
 * layers N > 3 skin depths thick (SolverExtension.cpp:509-541). SGBC tags on the domain boundary
 * become SMA faces (upwind_alpha 1 only); SGBC runs with evolution_operator "global" only. */
int dgtd_case_sgbc(const dgtd_case* c, dgtd_sgbc_stack* stacks, dgtd_sgbc_layer* layers, int32_t* face_stack);

/* The automatic time step a run of the case takes when solver_options.time_step is 0: the
 * reference's estimate for the case's evolution operator (Solver::estimateTimeStep,
 * Solver.cpp:289-345; global: base / 0.8, maxwell: base, hesthaven: cfl / (max Fscale p^2)),
 * from the case's mesh on the host (no device needed). */
int dgtd_case_auto_dt(const dgtd_case* c, double* dt);
/* Views into the case's tables (valid while the case lives). */
int dgtd_case_mesh(const dgtd_case* c, dgtd_mesh_desc* mesh);
int dgtd_case_planewaves(const dgtd_case* c, dgtd_planewave* out, int32_t capacity);
int dgtd_case_point_probes(const dgtd_case* c, double* h_points);
/* Surface s: its faces [n][3] (winding normal outwards); *n_faces gets the count (faces may be NULL). */
int dgtd_case_surface(const dgtd_case* c, int32_t s, int32_t* faces, int64_t* n_faces);
/* Initial fields at given nodes: h_xyz [3][n] -> h_state [6][n] (nodal projection). */
int dgtd_case_initial_state(const dgtd_case* c, const double* h_xyz, int64_t n, double* h_state);
/* Run the case to its final time on the GPU (reference Solver::run loop) with
 * point probes recorded at their intervals; h_state (may be NULL) gets the final
 * state (reference layout). */
int dgtd_case_run(const dgtd_case* c, const dgtd_case_run_opts* opts, double* h_state, dgtd_case_result* result);

/* ---- serving: continuous batching of independent solves ------------------------
 *
 * The reference runs one case per process (driver::buildSolverJson +
 * Solver::run, src/driver/driver.cpp:1545, src/solver/Solver.cpp:483-533). The
 * server runs many such solves at once on one GPU: each request is one
 * Solver::run of its own mesh, order, plane wave and final time, with classical
 * RK4 on the plain FP64 form or the single-instance FP32 form (the same
 * arithmetic as dgtd_op_step of that form, so a result is bit-identical alone
 * and in the mix). Requests are admitted as
 * device memory (a fixed budget, allocated once when the server starts) and
 * slots free up; every active request of one order advances in the same
 * kernel launches. Three host threads: admission (mesh tables, memory
 * reservation, upload), engine (launches), retirement (result download). */

#define DGTD_SERVER_MAX_ACTIVE 128

#define DGTD_REQ_QUEUED 0   /* submitted, waiting for memory */
#define DGTD_REQ_ACTIVE 1   /* uploaded / stepping */
#define DGTD_REQ_DONE 2
#define DGTD_REQ_FAILED 3

typedef struct dgtd_server dgtd_server;

typedef struct dgtd_server_opts {
    int64_t memory_budget;    /* device bytes for request regions, allocated at create (> 0) */
    int32_t max_active;       /* requests stepping at once, 1..DGTD_SERVER_MAX_ACTIVE */
    int32_t steps_per_round;  /* steps per active request between admission checks (>= 1) */
    int32_t device;           /* CUDA device ordinal */
    int32_t precision;        /* DGTD_FP64 (plain form) or DGTD_FP32 (single-instance FP32 form) */
} dgtd_server_opts;

typedef struct dgtd_request {
    const dgtd_mesh_desc* mesh;     /* copied by dgtd_server_submit */
    int32_t order;                  /* 1..6 */
    double alpha;                   /* upwind coefficient */
    const dgtd_planewave* waves;    /* batch index must be 0; may be NULL with n_waves = 0 */
    int32_t n_waves;                /* <= 8 */
    const double* h_init;           /* initial state, reference layout (6*K*Np); NULL = zero fields */
    double t0;
    double final_time;
    double dt;                      /* > 0: step size; <= 0: dgtd_op_estimate_dt at cfl */
    double cfl;
} dgtd_request;

typedef struct dgtd_request_stats {
    int32_t status;        /* DGTD_REQ_* */
    int32_t order;
    int64_t n_elements;
    int64_t state_len;     /* 6*K*Np */
    int64_t steps;         /* RK4 steps taken */
    int64_t region_bytes;  /* device bytes the request held */
    double dt;
    double t_submit;       /* seconds on the server clock (since create) */
    double t_admit;        /* region reserved and uploaded */
    double t_first_launch;
    double t_done;         /* result on the host */
    int32_t unstable;      /* 1: the final state's L2 norm was not finite or above 1e20 (the
                              instability detector of Solver::run, Solver.cpp:500-516, applied to
                              the downloaded result; a warning is printed on stderr) */
} dgtd_request_stats;

typedef struct dgtd_server_stats {
    int64_t submitted, completed, failed;
    int64_t active, queued;
    int64_t stage_launches;        /* stage kernels launched */
    int64_t slot_stage_updates;    /* sum over stage launches of the requests they advanced */
    int64_t max_active_seen;
    int64_t bytes_in_use, peak_bytes_in_use, memory_budget;
    int64_t dof_updates;           /* sum over requests of 6*K*Np per step taken */
} dgtd_server_stats;

/* Start a server (allocates the memory budget on the device, starts its threads). */
int dgtd_server_create(const dgtd_server_opts* opts, dgtd_server** out);
/* Stop the threads, fail requests not yet done, release all memory. */
void dgtd_server_destroy(dgtd_server* s);
/* Queue a request (inputs are copied; returns at once). DGTD_ERR_INVALID for a
 * malformed request; a request larger than the whole budget fails later with
 * DGTD_REQ_FAILED. */
int dgtd_server_submit(dgtd_server* s, const dgtd_request* req, int64_t* id_out);
/* Wait up to timeout_s seconds (< 0: forever) for request `id`. On DGTD_OK the
 * final state is copied to h_state (if not NULL; 6*K*Np doubles), *stats is
 * filled (if not NULL) and the request is released. DGTD_ERR_TIMEOUT leaves it
 * pending; a failed request returns DGTD_ERR_CUDA or DGTD_ERR_NOMEM with its
 * message in dgtd_last_error() and is released. */
int dgtd_server_wait(dgtd_server* s, int64_t id, double timeout_s, double* h_state, dgtd_request_stats* stats);
/* Status of a request without waiting (stats->status). */
int dgtd_server_query(dgtd_server* s, int64_t id, dgtd_request_stats* stats);
int dgtd_server_get_stats(dgtd_server* s, dgtd_server_stats* out);

/* Host-side range allocator the server carves request regions from (first fit,
 * neighbours merged on release); exported so its bookkeeping can be tested
 * without a GPU. */
typedef struct dgtd_arena dgtd_arena;
int dgtd_arena_create(int64_t capacity, int64_t align, dgtd_arena** out);
void dgtd_arena_destroy(dgtd_arena* a);
int64_t dgtd_arena_alloc(dgtd_arena* a, int64_t bytes);     /* offset, or -1 if no range fits */
int dgtd_arena_release(dgtd_arena* a, int64_t offset);      /* DGTD_OK or DGTD_ERR_INVALID */
int dgtd_arena_usage(const dgtd_arena* a, int64_t* in_use, int64_t* largest_free, int64_t* n_free_ranges);

/* ---- host-only mesh helpers (no GPU needed) ---------------------------------- */

/* Build the reference-element and mesh tables on the host only (the
 * once-per-mesh part of dgtd_op_create, no device allocation) and report them
 * in *info: validates a mesh description (connectivity, orientation, boundary
 * and TF/SF faces) without a GPU. */
int dgtd_mesh_validate(const dgtd_mesh_desc* mesh, const dgtd_op_opts* opts, dgtd_op_info* info);

/* Structured box mesh: n[3] cells on [lo,hi], each hex split into 6 tetrahedra
 * around its (0,0,0)-(1,1,1) diagonal (the split the reference's tests get from
 * Mesh::MakeCartesian3D(..., TETRAHEDRON), Solver3DTest.cpp:36). Cells in
 * [hole_lo, hole_hi) are removed (their surface gets hole_bc); cells in
 * [tf_lo, tf_hi) form the total-field region (its surface becomes TF/SF faces). */
typedef struct dgtd_box_spec {
    int32_t n[3];
    double lo[3], hi[3];
    int32_t hole_lo[3], hole_hi[3];
    int32_t tf_lo[3], tf_hi[3];
    int32_t outer_bc, hole_bc;
} dgtd_box_spec;

int dgtd_box_mesh_size(const dgtd_box_spec* spec, int64_t* n_vertices, int64_t* n_elements,
                       int64_t* n_bdr_faces, int64_t* n_tfsf_faces);
int dgtd_box_mesh_fill(const dgtd_box_spec* spec, double* vertices, int32_t* elements, int32_t* bdr_faces,
                       int32_t* bdr_codes, int32_t* tfsf_faces);

/* Reference-element tables of the product (host only), for known-answer
 * tests against the reference's element-matrix tests
 * (test/hesthavenComparison/Hesthaven3DTest.cpp:77-152, 232-265).
 * Arrays: r,s,t [Np]; Dr,Ds,Dt,Minv [Np*Np]; lift [Np*4*Nfp]; fmask [4*Nfp]
 * (row-major, Hesthaven (-1,1) reference tetrahedron). Any pointer may be NULL. */
int dgtd_ref_tet(int32_t order, double* r, double* s, double* t, double* Dr, double* Ds, double* Dt,
                 double* Minv, double* lift, int32_t* fmask);

/* Device self-check of the tensor-core (tcgen05, kind::tf32) building blocks the
 * batched form uses: D[128 x 48] = A[128 x k] * B[48 x k]^T in 3xTF32 on one CTA.
 * h_a [128*k], h_b [48*k], h_d [128*48] host, row-major; k a multiple of 8, <= 96.
 * *status: 0 ok, 2 the tensor-core completion wait timed out. */
int dgtd_tc_selftest(const float* h_a, const float* h_b, float* h_d, int32_t k, int32_t* status);

#ifdef __cplusplus
}
#endif

#endif /* DGTD_GB300_H */
