// matfree.cuh -- tables and state of the mixed-precision matrix-free SIMP
// operator (structured HEX8 grids), shared by the single-problem solve, the
// batched solver and the request loop.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "hex8_factored.cuh"
#include "mg_internal.h"

namespace mg {

// Owned-node brick edge; a brick reads the (kBN+2)^3 node halo and evaluates
// the (kBN+1)^3 elements around its kBN^3 owned nodes.
constexpr int kBN = 8;
constexpr int kBE = kBN + 1;
constexpr int kBU = kBN + 2;
constexpr int kNEL = kBE * kBE * kBE;          // 729 elements per brick
constexpr int kNTILE = (kNEL + 127) / 128;     // 6 MMA tiles of 128 elements
constexpr int kChunk = 4096;                   // dofs per vector-kernel chunk (four float4 per thread)
constexpr int kMapsPerProblem = 6;             // z, p0, p1, E, mg x, mg d (column operator boxes)
// Column operator: a column owns kCX x kCY nodes in x, y and up to kCZ node
// planes in z; it streams through its element planes (8 x 16 elements each,
// one M = 128 tensor-core tile per plane).
constexpr int kCX = 7;
constexpr int kCY = 15;
constexpr int kCZ = 32;   // most node planes per column
constexpr int kMaxLevels = 8;                  // multigrid levels per design
constexpr int kBottomMaxLevels = 6;            // levels of a bottom chain (one-CTA or cluster kernel)

// level table of the cluster bottom kernel (one chain, one cluster)
struct ClusterLevel {
    int NX, NY, NZ, nx, ny, nz;
    int pitch, pitch_e;
    int64_t dof_off, elem_off;
    int chunk;                // nodes per CTA (CTA r owns nodes [r chunk, (r + 1) chunk))
    int s_dinv, s_E, s_vec;   // shared-memory offsets (floats): D^-1 and E of the level, the CTA's slabs
    int NXY;                  // NX NY
    float rNX, rNXY, rchunk;  // 1 / NX, 1 / NXY, 1 / chunk: n / d = trunc((n + 1/2) (1 / d)) (checked on the host)
};
struct ClusterChain {
    int m, root, s_stage, pad;
    ClusterLevel L[kBottomMaxLevels];
};

// Padded vector layout of one problem: node (i,j,k), component c lives at
//   dof_off + (k NY + j) pitch + 3 i + c,   pitch = roundup(3 NX, 4)
// so that every (j,k) row starts on a 16-byte boundary (TMA row strides).
// Element moduli: elem_off + (k ny + j) pitch_e + i, pitch_e = roundup(nx, 4).
struct MfProblem {
    int nx, ny, nz;       // elements
    int NX, NY, NZ;       // nodes
    int pitch, pitch_e;
    int64_t n_dofs;       // 3 NX NY NZ
    int64_t n_pad;        // pitch NY NZ
    int64_t dof_off;      // offset into the concatenated padded dof vectors
    int64_t elem_off;     // offset into the padded element tables (E32, Edf, dE64)
    int64_t node_off;     // offset into the node Dirichlet masks (unpadded)
    int brick_begin, brick_count;
    int chunk_begin, chunk_count;
    int col_begin, col_count;
    int col_z;            // node planes per column (kCZ or fewer for small grids)
    int fac_begin, fac_count;
    int fac_z;            // node planes per tile of the factored CUDA-core operator
    int share_elems;      // >= 0: reuse the element tables of that problem (load cases)
    int level;            // multigrid level (0 = the design's own grid)
    int root;             // level-0 problem whose solver state drives this one
    int coarse, fine;     // neighbouring levels (-1 if none)
    int bottom;           // 1: solved inside the one-CTA bottom V-cycle of its chain
};

struct MfBrick {
    int prob;
    int16_t bx, by, bz, pad;
};

struct MfCol {
    int prob;
    int16_t cx, cy, cz, pad;
};

struct MfChunkDesc {
    int prob;
    int pad;
    int64_t begin, end;  // absolute padded dof range
};

// Per-problem solver state (device resident).  Each level-0 problem moves
// through the refinement phases on the device, independently of the others:
//   RESID (FP64 r = f - K u, stop test) -> INIT (inner CG start on r/||r||)
//   -> CG (inner iterations until the inner tolerance) -> RESID (after u += d)
//   ... -> FIN.
// `done` is 1 whenever the problem is not iterating its inner CG; the operator,
// vector and multigrid kernels skip such problems.
constexpr int kPhaseResid = 0;
constexpr int kPhaseInit = 1;
constexpr int kPhaseCG = 2;
constexpr int kPhaseFin = 3;

struct MfState {
    double rz, rr, pq, alpha, beta, bb, tol2;
    double rr64, ff64, scale;
    int iter, done, status, maxit;
    int total_iter, refine, ref_done, ref_status;
    int phase, first, u_zero, pad1; // first: the next dot_rz starts the inner CG (beta = 0);
                                    // u_zero: u is still 0 (the residual is f)
    unsigned cnt_apply, cnt_update, cnt_res, pad;
};

struct MfBatch {
    int n_probs = 0;
    int n_bricks = 0;
    int n_chunks = 0;
    int64_t n_pad = 0, n_elem_pad = 0, n_nodes = 0;
    std::vector<MfProblem> h_probs;
    std::vector<MfBrick> h_bricks;
    std::vector<MfChunkDesc> h_chunks;
    MfProblem *probs = nullptr;
    MfBrick *bricks = nullptr;
    MfCol *cols = nullptr;
    std::vector<MfCol> h_cols;
    int n_cols = 0;
    std::vector<int> lvl_col_lo, lvl_col_hi;
    double *col_part = nullptr;   // per-column partial of p.q
    uint32_t *Bop2 = nullptr;     // K0 as the column operator's four (dy, dz) B tiles
    MfCol *fac_tiles = nullptr;   // tiles of the factored CUDA-core operator (cx, cy, cz)
    CUtensorMap *fac_maps = nullptr;  // its tensor maps per problem (node vectors, moduli)
    std::vector<MfCol> h_fac_tiles;
    std::vector<int> lvl_fac_lo, lvl_fac_hi;
    FacK<float> fac32{};          // K0 in the per-axis sum/difference basis
    FacK<double> fac64{};
    FacK<dfloat> facdf{};         // fac64 as double-float pairs (the outer residual)
    FacK2 fac2{};                 // fac32 as (k, k) pairs for the packed FP32x2 kernels
    MfChunkDesc *chunks = nullptr;
    MfState *states = nullptr;
    MfState *states_host = nullptr;  // pinned
    int *err_host = nullptr;         // pinned copy of *err (step_begin / step_end)
    CUtensorMap *tmaps = nullptr;    // kMapsPerProblem per problem
    // element / node tables
    float *E32 = nullptr;
    dfloat *Edf = nullptr;      // the moduli as double-float pairs (the outer residual)
    double *dE64 = nullptr;
    uint8_t *node_fix = nullptr;
    // FP32 inner CG vectors (padded layout)
    float *x = nullptr, *r = nullptr, *z = nullptr, *p0 = nullptr, *p1 = nullptr, *q = nullptr,
          *dinv = nullptr, *xdbg = nullptr;
    // multigrid vectors (padded layout, every level): rhs, solution, Chebyshev
    // direction, operator output, residual
    float *mb = nullptr, *mx = nullptr, *md = nullptr, *my = nullptr, *mr = nullptr;
    int n_fine = 0;             // level-0 problems (the designs); problems are ordered by level
    int n_levels = 1;
    std::vector<int> lvl_prob_lo, lvl_prob_hi, lvl_brick_lo, lvl_brick_hi, lvl_chunk_lo, lvl_chunk_hi;
    double cheb_lmax = 0.0;     // Gershgorin bound of D^-1 A (same on every level)
    // bottom V-cycle: the head (first bottom level) of every chain that has one
    std::vector<int> h_heads;
    int *heads = nullptr;
    // direct solve on a chain's coarsest grid (when it has at most kCoarseDirectMax
    // dofs): the FP32 inverse of its assembled operator per chain, at coarse_off[head]
    // (-1: Chebyshev smoothing instead); formed on the device whenever the moduli
    // change, coarse_ok[head] = 0 where that met a non-positive pivot (smoothing then)
    std::vector<int64_t> h_coarse_off;
    std::vector<int> h_head_root;   // level-0 problem of each chain
    int64_t *coarse_off = nullptr;
    float *coarse_inv = nullptr;
    int *coarse_ok = nullptr;
    int bottom_smem = 0;        // dynamic shared memory of the bottom kernel
    int bottom_cluster = 0;     // CTAs per chain of the cluster bottom kernel (0: one-CTA kernel)
    std::vector<ClusterChain> h_cl_chains;  // its per-chain level tables
    ClusterChain *cl_chains = nullptr;
    float *cl_k0 = nullptr;     // K0 and its regrouped copy in FP32
    // FP64 refinement vectors (padded layout)
    double *u64 = nullptr, *r64 = nullptr, *f64 = nullptr;
    double *brick_part = nullptr, *chunk_part = nullptr;
    int *err = nullptr;
    int *diag_list = nullptr;  // problem list of a partial Jacobi update, then its direct chains
    int *stage_host = nullptr;  // pinned staging of diag_list
    int64_t *sens_offs = nullptr, *sens_offs_host = nullptr;  // dC/drho output offsets (device, pinned)
    cudaEvent_t stage_ev = nullptr;  // its last copy
    bool stage_pending = false;
    // operator data
    double *K0 = nullptr;     // 24x24 FP64, node-interleaved element order
    double hx = 1, hy = 1, hz = 1, nu = 0.3;
    cudaGraphExec_t graph = nullptr;  // solver steps (see enqueue_step)
    std::vector<double> graph_key;    // parameters the graph was captured with
    long long graph_launches = 0;     // kernel nodes in the graph
    int enqueue_error = 0;            // an operator asked for a vector without a tensor map
    int apply_grid = 0, vec_grid = 0, col_grid = 0, fac_grid = 0;
    cudaStream_t stream = nullptr;
};

struct MfSolveParams {
    int precision;        // MG_MIXED_*
    double rtol;          // FP64 outer residual target
    double inner_rtol;    // FP32 inner CG tolerance
    int max_iterations;   // inner cap per refinement
    int max_refinements;
    int graph_chunk;
    double timeout_s;
    int mg;               // 1: geometric multigrid V-cycle preconditioner, 0: Jacobi
    int smooth_deg;       // Chebyshev degree of the pre/post smoothers
    int coarse_deg;       // Chebyshev degree on the coarsest level
    int mg_operator = 0;  // multigrid level operator: 0 factored FP32 (CUDA cores), 1 tensor cores
    int vec_blocks_per_sm = 0;         // grid of the vector kernels (0 = 8 per SM)
    const uint8_t *active = nullptr;   // per level-0 problem: 0 = leave untouched (nullable)
};

// host-side element stiffness of an hx x hy x hz box at E = 1 in
// node-interleaved element order (dof 3a + c)
void hex8_box_stiffness(double hx, double hy, double hz, double nu, double K[576]);

// shapes: the designs' own grids (level 0); max_levels > 1 adds the coarse
// multigrid levels of every design (coarsening while all dims stay even);
// bottom_cluster: each chain's bottom V-cycle on a thread-block cluster from a
// larger level on (single-design solves; batches keep the one-CTA form, so a
// design's preconditioner is the same in every batch)
int mf_batch_init(MfBatch &b, const std::vector<MfProblem> &shapes, double hx, double hy,
                  double hz, double nu, cudaStream_t stream, int max_levels = kMaxLevels,
                  bool bottom_cluster = false);
void mf_batch_free(MfBatch &b);
// per-problem Dirichlet mask (per node, bit c = component c fixed) and load (unpadded host)
int mf_batch_set_bc(MfBatch &b, int i, const uint8_t *node_fix_host, const double *f_host);
// per-problem moduli from unpadded device arrays (E and dE/drho, n_elems each)
int mf_batch_set_moduli(MfBatch &b, int i, const double *E_dev, const double *dE_dev);
int mf_batch_solve(MfBatch &b, const MfSolveParams &prm, bool warm_start);
// stepping interface (mf_batch_solve and the request loop are built on it):
// prepare captures the step graph for prm; reset puts every problem at FIN;
// activate starts the listed level-0 problems at the FP64 residual (their
// Jacobi inverses are refreshed; u is zeroed unless warm_start); step runs one
// graph launch and refreshes states_host (synchronising); finish returns a
// FIN problem's status and zeroes u of a zero-load problem.
int mf_batch_prepare(MfBatch &b, const MfSolveParams &prm);
int mf_batch_reset_states(MfBatch &b);
int mf_batch_activate(MfBatch &b, const std::vector<int> &level0, bool warm_start);
int mf_batch_step(MfBatch &b);
// the same in two halves, so that several batches can run on the GPU at once:
// begin launches the step graph and the state copy, end waits for them
int mf_batch_step_begin(MfBatch &b);
int mf_batch_step_end(MfBatch &b);
int mf_batch_finish(MfBatch &b, int i);
// active (nullable, per level-0 problem): 0 = leave that problem's dc untouched
int mf_batch_compliance(MfBatch &b, double *compliance_host, double *dc_unpadded_dev,
                        const uint8_t *active = nullptr);
// u (padded, FP64) <-> unpadded node-interleaved device vector of problem i
int mf_batch_get_u(MfBatch &b, int i, double *u_dev);
int mf_batch_set_u(MfBatch &b, int i, const double *u_dev);
int mf_apply(MfBatch &b, int precision, const double *x_host, double *y_host, int prob);
int mf_launch_apply(MfBatch &b, int precision, int reps);

}  // namespace mg
