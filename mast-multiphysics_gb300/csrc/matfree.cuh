// matfree.cuh -- tables and state of the mixed-precision matrix-free SIMP
// operator (structured HEX8 grids), shared by the single-problem solve, the
// batched solver and the request loop.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "mg_internal.h"

namespace mg {

// Owned-node brick edge; a brick reads (kBN+2)^3 nodes and evaluates the
// (kBN+1)^3 elements around its kBN^3 owned nodes.
constexpr int kBN = 8;
constexpr int kBE = kBN + 1;
constexpr int kBU = kBN + 2;
constexpr int kNEL = kBE * kBE * kBE;          // 729 elements per brick
constexpr int kNTILE = (kNEL + 127) / 128;     // 6 MMA tiles of 128 elements
constexpr int kResStride = 25;                 // odd stride: conflict-free rows
constexpr int kChunk = 4096;                   // dofs per vector-kernel chunk

// One structured problem (a design evaluation x one load case) in a batch.
struct MfProblem {
    int nx, ny, nz;       // elements
    int NX, NY, NZ;       // nodes
    int64_t n_dofs;
    int64_t dof_off;      // offset into the concatenated dof vectors
    int64_t elem_off;     // offset into the element tables (E, dE)
    int64_t node_off;     // offset into the node Dirichlet masks
    int brick_begin, brick_count;
    int chunk_begin, chunk_count;
};

struct MfBrick {
    int prob;
    int16_t bx, by, bz, pad;
};

struct MfChunkDesc {
    int prob;
    int pad;
    int64_t begin, end;  // absolute dof range
};

// Per-problem solver state (device resident).
struct MfState {
    double rz, rr, pq, alpha, beta, bb, tol2;
    double rr64, ff64, scale;
    int iter, done, status, maxit;
    int total_iter, refine, ref_done, ref_status;
    unsigned cnt_apply, cnt_update, cnt_res, pad;
};

struct MfBatch {
    int n_probs = 0;
    int n_bricks = 0;
    int n_chunks = 0;
    int64_t n_dofs = 0, n_elems = 0, n_nodes = 0;
    std::vector<MfProblem> h_probs;
    std::vector<MfBrick> h_bricks;
    std::vector<MfChunkDesc> h_chunks;
    MfProblem *probs = nullptr;
    MfBrick *bricks = nullptr;
    MfChunkDesc *chunks = nullptr;
    MfState *states = nullptr;
    MfState *states_host = nullptr;  // pinned
    // element / node tables
    float *E32 = nullptr;
    double *E64 = nullptr, *dE64 = nullptr;
    uint8_t *node_fix = nullptr;
    // FP32 inner CG vectors
    float *x = nullptr, *r = nullptr, *z = nullptr, *p0 = nullptr, *p1 = nullptr, *q = nullptr,
          *dinv = nullptr;
    // FP64 refinement vectors
    double *u64 = nullptr, *r64 = nullptr, *f64 = nullptr;
    double *brick_part = nullptr, *chunk_part = nullptr;
    int *err = nullptr;
    // operator data
    uint32_t *Bop_tf32 = nullptr, *Bop_bf16 = nullptr;  // K0 in the UMMA smem layout
    double *K0 = nullptr;                               // 24x24 FP64, node-interleaved
    double hx = 1, hy = 1, hz = 1, nu = 0.3;
    cudaGraphExec_t graph = nullptr;
    int graph_prec = -1, graph_chunk = 0;
    int apply_grid = 0, vec_grid = 0;
    cudaStream_t stream = nullptr;
    bool owns_stream = false;
};

struct MfSolveParams {
    int precision;        // MG_MIXED_TF32 / MG_MIXED_BF16
    double rtol;          // FP64 outer residual target
    double inner_rtol;    // FP32 inner CG tolerance
    int max_iterations;   // inner cap per refinement
    int max_refinements;
    int graph_chunk;
    double timeout_s;
};

// host-side element stiffness of an hx x hy x hz box at E = 1 in
// node-interleaved element order (dof 3a + c)
void hex8_box_stiffness(double hx, double hy, double hz, double nu, double K[576]);

int mf_batch_init(MfBatch &b, const std::vector<MfProblem> &shapes, double hx, double hy,
                  double hz, double nu, cudaStream_t stream);
void mf_batch_free(MfBatch &b);
// per-problem Dirichlet masks, loads and moduli
int mf_batch_set_problem(MfBatch &b, int i, const uint8_t *node_fix_host, const double *f_host,
                         const double *E_dev, const double *dE_dev);
int mf_batch_solve(MfBatch &b, const MfSolveParams &prm, bool warm_start);
int mf_batch_compliance(MfBatch &b, double *compliance_host, double *dc_dev_all);
int mf_apply(MfBatch &b, int precision, const float *x, float *y);

}  // namespace mg
