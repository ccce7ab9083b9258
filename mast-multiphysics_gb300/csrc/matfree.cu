// matfree.cu -- mixed-precision matrix-free SIMP operator on the 5th-generation
// tensor cores, FP32 inner CG and FP64 iterative refinement.
//
// Operator: y = sum_e E_e P_e^T K0 P_e u on a structured HEX8 grid (every
// element shares the reference stiffness K0 of StructuralElement3D,
// src/elasticity/solid_element_3d.cpp:135-423, scaled by the SIMP modulus of
// examples/structural/example_6/example_6.cpp:100-137).  Dirichlet dofs are
// eliminated (identity rows, zero columns) as in the plain form; they are
// marked by a zero Jacobi inverse, which keeps r, z and p zero there.
//
// Brick kernel (one CTA per 8x8x8 block of owned nodes, persistent grid,
// two CTAs per SM):
//   1. one thread issues three TMA tile loads (cp.async.bulk.tensor.3d) into
//      shared memory: the (8+2)^3 node halo of z and of p_old, and the 9^3
//      element moduli around the owned nodes; out-of-grid parts arrive as 0;
//   2. per 128-element tile, all threads write the element displacement rows
//      U = z + beta p_old (128 x 24) as TF32 or BF16 in the canonical
//      no-swizzle K-major UMMA layout (the split variants also write the
//      rounding remainder U_lo), and one thread issues tcgen05.mma:
//      D(128 x 32, FP32, TMEM) = U K0^T [+ U_lo K0^T + U K0_lo^T];
//      two A buffers and two TMEM accumulators let tile t's MMA run while
//      tile t-1 is drained;
//   3. tcgen05.ld drains D, each row is scaled by E_e (the rho^p epilogue) and
//      parked in a 128-row shared buffer;
//   4. every owned dof adds the contributions of its (up to 8) elements found
//      in that tile, in a fixed order, into a register accumulator: no atomics,
//      no colouring, deterministic, one global write per output dof.
// Elements in the one-element halo are evaluated by both neighbouring bricks
// (729 evaluations per 512 owned nodes).
//
// Reductions are per problem and deterministic: every brick (chunk) writes a
// partial and the last brick (chunk) of a problem -- found with a per-problem
// counter -- sums that problem's partials in index order.  A problem's result
// is therefore bitwise independent of which other problems share the batch.
#include <cstdlib>
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>

#include "matfree.cuh"

namespace mg {

namespace {

constexpr int kThreads = 256;

template <int P>
struct Prec {
    static constexpr bool kTf32 = (P == MG_MIXED_TF32 || P == MG_MIXED_TF32X3);
    static constexpr bool kSplit = (P == MG_MIXED_TF32X3 || P == MG_MIXED_BF16X3);
};

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// UMMA shared-memory descriptor, no swizzle, K-major canonical layout:
// 8-row x 16-byte core matrices; LBO = byte step between core matrices along K,
// SBO = byte step between 8-row groups; version field = 1 (sm_100 family).
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;  // base offset 0, LBO mode 0, layout type 0 (SWIZZLE_NONE)
}

// instruction descriptor: D F32, A/B K-major, N columns, M = 128
template <bool TF32, int N>
__host__ __device__ constexpr uint32_t umma_idesc() {
    return (1u << 4) |                   // D format F32
           ((TF32 ? 2u : 1u) << 7) |     // A: TF32 (kind::tf32) / BF16 (kind::f16)
           ((TF32 ? 2u : 1u) << 10) |    // B
           (((uint32_t)N >> 3) << 17) |  // N >> 3
           ((128u >> 4) << 24);          // M >> 4
}

template <bool TF32, int N>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                     uint32_t accumulate) {
    if (TF32) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
            ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(umma_idesc<TF32, N>()), "r"(accumulate));
    } else {
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
            ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(umma_idesc<TF32, N>()), "r"(accumulate));
    }
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Programmatic dependent launch: let the next kernel of the stream be scheduled
// now, then wait until the previous kernel has finished and its writes are
// visible (a no-op without a programmatic dependency).
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_enter() {
    pdl_trigger();
    pdl_wait();
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(mbar), "r"(phase)
        : "memory");
    return ok != 0;
}

// bounded wait: false after the iteration cap (the caller records the error)
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t phase) {
    for (int i = 0; i < (1 << 22); i++)
        if (mbar_try_wait(mbar, phase)) return true;
    return false;
}

// 3D TMA tile load global -> shared, completion on an mbarrier
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            int z, uint32_t mbar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(mbar)
        : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

// libMesh HEX8 local node a -> corner bits
__host__ __device__ __forceinline__ void corner_bits(int a, int &dx, int &dy, int &dz) {
    dx = ((a + 1) >> 1) & 1;
    dy = (a >> 1) & 1;
    dz = (a >> 2) & 1;
}
__host__ __device__ __forceinline__ int corner_index(int dx, int dy, int dz) {
    return dz * 4 + (dy ? (dx ? 2 : 3) : (dx ? 1 : 0));
}

__device__ __forceinline__ int64_t dof_index(const MfProblem &P, int gx, int gy, int gz, int c) {
    return P.dof_off + ((int64_t)gz * P.NY + gy) * P.pitch + 3 * gx + c;
}

// --------------------------------------------------------------- block helpers
__device__ __forceinline__ double block_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < kThreads / 32; i++) s += sh[i];
    return s;  // valid in thread 0
}

// FP32 warp sums, FP64 across the block's warps; valid in thread 0
__device__ __forceinline__ double block_sum_f(float v, double *sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sh[w] = (double)v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < kThreads / 32; i++) s += sh[i];
    return s;
}

// fixed-order sum of part[begin .. begin+count) over the block; valid in thread 0
__device__ __forceinline__ double ordered_sum(const double *part, int begin, int count) {
    __shared__ double tree[kThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < count; i += kThreads) s += __ldcg(part + begin + i);
    __syncthreads();
    tree[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) tree[threadIdx.x] += tree[threadIdx.x + w];
        __syncthreads();
    }
    return tree[0];
}

__device__ __forceinline__ bool is_bad(double x) { return !isfinite(x); }

// ----------------------------------------------------------- column operator
// y = sum_e E_e P_e^T K0 P_e x by columns of owned nodes (kCX x kCY nodes in x,
// y; up to kCZ node planes in z), streamed plane by plane.  The A operand of
// the tensor-core MMA is never assembled: the halo nodes of each plane are
// converted once into 16-byte node records (x, y, z, 0 in TF32; x, y, z and five
// zeros in BF16), and the MMA reads them in place.  An element plane holds 8 x 16
// elements, one M = 128 tile: row r = ey * 8 + ex; the eight rows of a core
// matrix are eight x-consecutive elements (nodes 16 bytes apart), the 16 row
// groups are the 16 element rows (stride of a node row).  One MMA per corner
// pair (dx = 0, 1 at fixed dy, dz) uses K chunks 16 bytes apart (the node and
// its x-neighbour), so the element operator is 4 MMAs per product (3 products
// in the split forms) against four B tiles cut from K0.
//
// The cost of one tcgen05.mma (M = 128, K = 8 TF32) grows little with N up to
// 64 (46, 48, 64, 128 cycles for N = 32, 64, 128, 256, measured on the GB300), so
// the split forms issue the hi records against [K0_hi | K0_lo] as one N = 64 MMA
// and the lo records against K0_hi as an N = 32 MMA: 8 MMAs per element plane
// instead of 12.  The accumulator holds hi.K_hi + lo.K_hi in columns 0-31 and
// hi.K_lo in columns 32-63; the drain adds the two.
//
// Warp roles (no CTA-wide barrier inside the plane stream; every hand-off is an
// mbarrier with a bounded wait), two CTAs of 12 warps per SM:
//   warp 0      one thread issues the TMA loads of each node plane (z and, in the
//               CG step, p_old; the moduli of the element plane) into a ring;
//   warp 1      one thread issues the MMAs of element plane s once node planes s
//               and s+1 are converted, into one of four TMEM accumulators;
//   warps 2-7   convert a node plane into the operand records (hi and lo parts)
//               and an FP32 copy u of the owned nodes (with p = z + beta p_old
//               fused), plus the plane's moduli, into rings;
//   warps 8-11  drain: thread = element (TMEM lane), reads its 24 results, scales
//               by E_e, sums the corner results into nodes (x: warp shuffle, y:
//               shuffle and, at the warp's first row, the previous warp's last row
//               through shared memory; z: the top corners of plane s-1 carried in
//               registers) and writes node plane s of y (and p_new) -- every node
//               sum in a fixed order, deterministic and atomic-free.
// The column sequence is chosen by the TMA thread alone and travels with the data
// (a record per ring slot), ending with a sentinel plane.
constexpr int kColThreads = 384;
constexpr int kColCtas = 2;                   // CTAs per SM
constexpr int kCConvWarps = 6;                // warps 2-7
constexpr int kCDrain0 = 2 + kCConvWarps;     // first drain warp (8: TMEM lane quarter = warp % 4)
constexpr int kCPX = kCX + 2;                 // 9 nodes per plane row
constexpr int kCPY = kCY + 2;                 // 17 node rows per plane
constexpr int kCPN = kCPX * kCPY;             // 153 nodes per plane
constexpr int kCPB = kCPN * 16;               // 2448 bytes per converted plane (one part)
constexpr int kCRawX = 32;                    // TMA node box: 32 floats x 17 rows x 1 plane
constexpr int kCRawNode = kCRawX * kCPY * 4;  // 2176
constexpr int kCRawE = 12 * 16 * 4;           // E box: 12 elements x 16 rows x 1 plane = 768
constexpr int kCRawSlot = 2 * kCRawNode + kCRawE;  // 5120 (z, p_old, E)
constexpr int kCNR = 4;                       // TMA ring slots
constexpr int kCNC = 6;                       // operand-record ring slots (hi | lo)
constexpr int kCNU = 8;                       // u / E ring slots (the drain's inputs)
constexpr int kCNT = 4;                       // TMEM accumulators (64 columns each)
constexpr int kCTCols = 64;                   // TMEM columns per accumulator
constexpr int kCOwn = kCX * kCY;              // 105 owned nodes per plane
constexpr int kCUSlot = kCOwn * 16 + 128 * 4; // u of the owned nodes as (x, y, z, -) + 128 moduli = 2192
constexpr int kCConvFloats = kCPN * 3;        // 459 values per node plane
constexpr int kCConvThreads = 32 * kCConvWarps;
constexpr int kCConvRounds = (kCConvFloats + kCConvThreads - 1) / kCConvThreads;  // 3
constexpr int kCXch = 4 * 8 * 8;              // exchange slot: 4 warps x 8 lanes x (6 + 2 pad) floats

constexpr int kC_OffB = 0;                                          // 4 B tiles x 2 KB: [K_hi | K_lo]
constexpr int kC_OffConv = 8192;                                    // kCNC x (hi, lo) records
constexpr int kC_OffRaw = (kC_OffConv + kCNC * 2 * kCPB + 127) / 128 * 128;  // TMA ring
constexpr int kC_OffU = kC_OffRaw + kCNR * kCRawSlot;               // u / E ring
constexpr int kC_OffX = kC_OffU + kCNU * kCUSlot;                   // y-exchange, 2 slots
constexpr int kC_OffMeta = kC_OffX + 2 * kCXch * 4;                 // plane records (int4)
constexpr int kC_OffRed = kC_OffMeta + (kCNR + kCNC + kCNU) * 16;   // column partials [2][4]
constexpr int kC_OffBar = kC_OffRed + 64;                           // mbarriers
// barriers: raw full/empty, conv full/empty, u full/empty, tmem full/empty, xch[2], red[2], fin
constexpr int kCBarRawFull = 0, kCBarRawEmpty = kCBarRawFull + kCNR, kCBarConvFull = kCBarRawEmpty + kCNR,
              kCBarConvEmpty = kCBarConvFull + kCNC, kCBarUFull = kCBarConvEmpty + kCNC,
              kCBarUEmpty = kCBarUFull + kCNU, kCBarTFull = kCBarUEmpty + kCNU, kCBarTEmpty = kCBarTFull + kCNT,
              kCBarXch = kCBarTEmpty + kCNT, kCBarRed = kCBarXch + 2, kCBarFin = kCBarRed + 2,
              kCBarCount = kCBarFin + 1;
constexpr int kC_OffFlags = kC_OffBar + kCBarCount * 8;             // tmem slot, abort flag
constexpr int kColSmem = kC_OffFlags + 16;
static_assert(kC_OffRaw % 128 == 0 && kCRawSlot % 128 == 0 && kCRawNode % 128 == 0, "TMA destinations");
static_assert(kC_OffConv % 16 == 0 && kCPB % 16 == 0 && kC_OffU % 16 == 0 && kCUSlot % 16 == 0, "alignment");
static_assert(kC_OffMeta % 16 == 0 && kC_OffBar % 8 == 0, "alignment");
static_assert(kColCtas * (kColSmem + 1024) <= 228 * 1024, "CTAs per SM");
static_assert(kCNT * kCTCols * kColCtas <= 512, "TMEM columns of the CTAs on an SM");
static_assert(kColThreads == 32 * (kCDrain0 + 4), "warp roles");

// bounded mbarrier wait that also gives up when another role has set the CTA's
// abort flag; a wait that runs out of polls sets the flag
__device__ __forceinline__ bool col_wait(uint32_t mbar, uint32_t phase, volatile int *abort_flag) {
    for (int i = 0; i < (1 << 22); i++) {
        if (mbar_try_wait(mbar, phase)) return true;
        if ((i & 63) == 63 && *abort_flag) return false;
    }
    *abort_flag = 1;
    return false;
}

// columns [taddr, taddr + 24) of the warp's 32 TMEM lanes, one wait for both loads
__device__ __forceinline__ void tmem_ld24(uint32_t taddr, float (&v)[24]) {
    uint32_t r[24];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
          "=r"(r[23])
        : "r"(taddr + 16));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 24; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

// Columns col_lo .. col_hi-1; the input vector is tensor map `in_slot`.
// MODE 1: CG step, gathered u = z + beta p_old (z = in_slot, p_old = map 1 +
//         parity), p_new (owned) = u, q = A u, per-problem alpha = rz / (p.q).
// MODE 2: y = rhs - A x.   MODE 3: y = A x.   (Both 0 on Dirichlet dofs.)
// A wait that times out sets bit 1 (tensor-core hand-offs) or bit 2 (data
// hand-offs) of *err and ends the block after its copies and MMAs have landed.
template <int PREC, int MODE>
__global__ void __launch_bounds__(kColThreads, kColCtas) mf_col_kernel(
    const MfProblem *__restrict__ probs, const MfCol *__restrict__ cols, int col_lo, int col_hi, int sel,
    const CUtensorMap *__restrict__ tmaps, int in_slot, int parity, const uint32_t *__restrict__ Bop2,
    const float *__restrict__ dinv, const float *__restrict__ rhs, float *__restrict__ p0,
    float *__restrict__ p1, float *__restrict__ y, MfState *states, double *__restrict__ col_part,
    int *err) {
    // the prologue (barriers, TMEM, the constant B tiles, the zeroed records) overlaps
    // the previous kernel; everything after pdl_wait may read its results
    pdl_trigger();
    using PR = Prec<PREC>;
    extern __shared__ __align__(1024) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int4 *meta_raw = reinterpret_cast<int4 *>(smem + kC_OffMeta);
    int4 *meta_conv = meta_raw + kCNR;
    int4 *meta_u = meta_conv + kCNC;
    double *red = reinterpret_cast<double *>(smem + kC_OffRed);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + kC_OffFlags);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + kC_OffFlags + 4);
    const uint32_t bar0 = smem_u32(smem + kC_OffBar);
    auto bar = [&](int i) -> uint32_t { return bar0 + 8u * (uint32_t)i; };
    float *p_new = (MODE == 1) ? (parity ? p0 : p1) : nullptr;

    if (tid == 0) {
        for (int k = 0; k < kCNR; k++) {
            mbar_init(bar(kCBarRawFull + k), 1);
            mbar_init(bar(kCBarRawEmpty + k), kCConvWarps);
        }
        for (int k = 0; k < kCNC; k++) {
            mbar_init(bar(kCBarConvFull + k), kCConvWarps);
            mbar_init(bar(kCBarConvEmpty + k), 1);  // an MMA commit
        }
        for (int k = 0; k < kCNU; k++) {
            mbar_init(bar(kCBarUFull + k), kCConvWarps);
            mbar_init(bar(kCBarUEmpty + k), 4);     // the four drain warps
        }
        for (int k = 0; k < kCNT; k++) {
            mbar_init(bar(kCBarTFull + k), 1);
            mbar_init(bar(kCBarTEmpty + k), 4);
        }
        for (int k = 0; k < 2; k++) {
            mbar_init(bar(kCBarXch + k), 4);
            mbar_init(bar(kCBarRed + k), 4);
        }
        mbar_init(bar(kCBarFin), 1);
        *abort_flag = 0;
    }
    if (warp == 1) tmem_alloc(smem_u32(tslot), kCNT * kCTCols);
    {
        // B tiles in global memory: [tf32 hi 1024 | tf32 lo 1024 | bf16 hi 1024 | bf16 lo 1024]
        // words, tile t at 256 t in each part; in shared memory tile t at 512 t words as
        // [hi 256 | lo 256]: N = 64 rows, the lo rows one SBO step after the hi rows
        const uint32_t *src = Bop2 + (PR::kTf32 ? 0 : 2048);
        uint32_t *dst = reinterpret_cast<uint32_t *>(smem + kC_OffB);
        for (int i = tid; i < 2048; i += kColThreads) {
            const int part = i >> 10, t = (i >> 8) & 3, w = i & 255;
            dst[t * 512 + part * 256 + w] = src[i];
        }
        // node records: the unused lanes stay 0 (B has zero rows there; 0 x NaN is NaN)
        uint32_t *conv = reinterpret_cast<uint32_t *>(smem + kC_OffConv);
        for (int i = tid; i < kCNC * 2 * kCPB / 4; i += kColThreads) conv[i] = 0u;
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tslot;
    pdl_wait();

    if (warp == 0) {
        // ------------------------------------------------------------ TMA producer
        if (lane == 0) {
            uint32_t k = 0;
            int last_issue[kCNR] = {-1, -1, -1, -1};
            auto usable = [&](int ci) {
                const MfProblem &Q = probs[cols[ci].prob];
                return !states[Q.root].done && !Q.bottom && (sel < 0 || sel == (Q.coarse < 0 ? 1 : 0));
            };
            bool ok = true;
            int ci = col_lo + blockIdx.x;
            while (ci < col_hi && !usable(ci)) ci += gridDim.x;
            for (; ci < col_hi && ok;) {
                const MfCol cl = cols[ci];
                const MfProblem &P = probs[cl.prob];
                const int x0 = cl.cx * kCX, y0 = cl.cy * kCY, z0 = cl.cz * P.col_z;
                const int z1 = min(z0 + P.col_z, P.NZ);
                const int S = z1 - z0 + 1;                      // element planes z0-1 .. z1-1
                const int xs = (3 * (x0 - 1)) & ~3, xe = (x0 - 1) & ~3;  // 16-byte aligned box starts
                const CUtensorMap *maps = tmaps + (size_t)cl.prob * kMapsPerProblem;
                for (int p = 0; p <= S; p++, k++) {
                    const int slot = (int)(k % kCNR);
                    if (!col_wait(bar(kCBarRawEmpty + slot), ((k / kCNR) & 1u) ^ 1u, abort_flag)) {
                        ok = false;
                        break;
                    }
                    meta_raw[slot] = make_int4(ci, p, S, 0);
                    uint8_t *raw = smem + kC_OffRaw + slot * kCRawSlot;
                    const uint32_t bytes = (MODE == 1 ? 2 : 1) * kCRawNode + (p < S ? kCRawE : 0);
                    mbar_expect_tx(bar(kCBarRawFull + slot), bytes);
                    tma_load_3d(smem_u32(raw), maps + in_slot, xs, y0 - 1, z0 - 1 + p, bar(kCBarRawFull + slot));
                    if (MODE == 1)
                        tma_load_3d(smem_u32(raw + kCRawNode), maps + 1 + parity, xs, y0 - 1, z0 - 1 + p,
                                    bar(kCBarRawFull + slot));
                    if (p < S)
                        tma_load_3d(smem_u32(raw + 2 * kCRawNode), maps + 3, xe, y0 - 1, z0 - 1 + p,
                                    bar(kCBarRawFull + slot));
                    last_issue[slot] = (int)k;
                }
                ci += gridDim.x;
                while (ci < col_hi && !usable(ci)) ci += gridDim.x;
            }
            if (ok) {
                // sentinel: no data, the stream ends
                const int slot = (int)(k % kCNR);
                if (col_wait(bar(kCBarRawEmpty + slot), ((k / kCNR) & 1u) ^ 1u, abort_flag)) {
                    meta_raw[slot] = make_int4(-1, 0, 0, 0);
                    mbar_arrive(bar(kCBarRawFull + slot));
                }
            }
            if (*abort_flag) {
                atomicOr(err, 2);
                // let the copies in flight land before the block exits
                for (int s = 0; s < kCNR; s++)
                    if (last_issue[s] >= 0) {
                        const uint32_t ph = ((uint32_t)last_issue[s] / kCNR) & 1u;
                        for (int i = 0; i < (1 << 22) && !mbar_try_wait(bar(kCBarRawFull + s), ph); i++) {
                        }
                    }
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t b_base = smem_u32(smem + kC_OffB), conv_base = smem_u32(smem + kC_OffConv);
            uint32_t es = 0;
            for (uint32_t k = 0;; k++) {
                const int cs = (int)(k % kCNC);
                if (!col_wait(bar(kCBarConvFull + cs), (k / kCNC) & 1u, abort_flag)) break;
                const int4 m = meta_conv[cs];
                if (m.x < 0) break;
                if (m.y >= 1) {
                    // element plane m.y - 1 from node planes k - 1 (dz = 0) and k (dz = 1)
                    const int ts = (int)(es % kCNT);
                    if (!col_wait(bar(kCBarTEmpty + ts), ((es / kCNT) & 1u) ^ 1u, abort_flag)) break;
                    fence_after();
                    const uint32_t d = tmem + (uint32_t)ts * kCTCols;
                    const int cprev = (int)((k - 1) % kCNC);
#pragma unroll
                    for (int st4 = 0; st4 < 4; st4++) {
                        const int dy = st4 & 1, dz = st4 >> 1;
                        const uint32_t a = conv_base + (dz ? cs : cprev) * 2 * kCPB + dy * kCPX * 16;
                        const uint64_t bd = umma_desc(b_base + st4 * 2048, 128, 256);
                        if (PR::kSplit) {
                            // hi records against [K_hi | K_lo] (columns 0-63), lo records
                            // against K_hi (columns 0-31)
                            umma<PR::kTf32, 64>(d, umma_desc(a, 16, kCPX * 16), bd, st4 ? 1u : 0u);
                            umma<PR::kTf32, 32>(d, umma_desc(a + kCPB, 16, kCPX * 16), bd, 1u);
                        } else {
                            umma<PR::kTf32, 32>(d, umma_desc(a, 16, kCPX * 16), bd, st4 ? 1u : 0u);
                        }
                    }
                    umma_commit(bar(kCBarTFull + ts));
                    umma_commit(bar(kCBarConvEmpty + cprev));             // node plane k - 1 is done
                    if (m.y == m.z) umma_commit(bar(kCBarConvEmpty + cs)); // the column's last node plane
                    es++;
                }
            }
            // every MMA issued has completed before the accumulators are freed
            umma_commit(bar(kCBarFin));
            for (int i = 0; i < (1 << 22) && !mbar_try_wait(bar(kCBarFin), 0u); i++) {
            }
            if (*abort_flag) atomicOr(err, 1);
        }
    } else if (warp < kCDrain0) {
        // ------------------------------------------------------------ converters
        const int ct = tid - 64;
        // per round: raw-box float index (ox added), record word, word of u (owned nodes)
        int src[kCConvRounds], dst[kCConvRounds], udst[kCConvRounds];
#pragma unroll
        for (int j = 0; j < kCConvRounds; j++) {
            const int i = ct + kCConvThreads * j;
            const int row = i / 27, kk = i - 27 * row, nx = kk / 3;
            src[j] = (i < kCConvFloats) ? row * kCRawX + kk : -1;
            dst[j] = (row * kCPX + nx) * 4 + kk % 3;  // node n, component c: word 4 n + c
            const bool owned = nx >= 1 && nx <= kCX && row >= 1 && row <= kCY;
            udst[j] = owned ? ((row - 1) * kCX + nx - 1) * 4 + kk % 3 : -1;
        }
        float beta = 0.0f;
        int ox = 0, oe = 0;
        for (uint32_t k = 0;; k++) {
            const int rs = (int)(k % kCNR), cs = (int)(k % kCNC), us = (int)(k % kCNU);
            bool ok = col_wait(bar(kCBarRawFull + rs), (k / kCNR) & 1u, abort_flag);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) break;
            const int4 m = meta_raw[rs];
            ok = col_wait(bar(kCBarConvEmpty + cs), ((k / kCNC) & 1u) ^ 1u, abort_flag) &&
                 col_wait(bar(kCBarUEmpty + us), ((k / kCNU) & 1u) ^ 1u, abort_flag);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) break;
            if (m.x >= 0) {
                if (m.y == 0) {
                    const MfCol cl = cols[m.x];
                    const int x0 = cl.cx * kCX;
                    ox = 3 * (x0 - 1) - ((3 * (x0 - 1)) & ~3);
                    oe = (x0 - 1) - ((x0 - 1) & ~3);
                    beta = (MODE == 1) ? (float)states[cl.prob].beta : 0.0f;
                }
                const float *rz = reinterpret_cast<const float *>(smem + kC_OffRaw + rs * kCRawSlot);
                const float *rp = rz + kCRawNode / 4;
                const float *re = rz + 2 * kCRawNode / 4;
                uint32_t *hi = reinterpret_cast<uint32_t *>(smem + kC_OffConv + cs * 2 * kCPB);
                uint32_t *lo = hi + kCPB / 4;
                float *u = reinterpret_cast<float *>(smem + kC_OffU + us * kCUSlot);
                // all loads first: the stores below cannot alias them, but the compiler
                // cannot tell, and would otherwise order each round after the last
                float vz[kCConvRounds], vp[kCConvRounds];
#pragma unroll
                for (int j = 0; j < kCConvRounds; j++) {
                    const int bo = (src[j] < 0 ? 0 : src[j]) + ox;
                    vz[j] = rz[bo];
                    vp[j] = (MODE == 1) ? rp[bo] : 0.0f;
                }
#pragma unroll
                for (int j = 0; j < kCConvRounds; j++) {
                    if (src[j] < 0) continue;
                    const float v = (MODE == 1) ? fmaf(beta, vp[j], vz[j]) : vz[j];
                    if (MODE == 1 && udst[j] >= 0) u[udst[j]] = v;
                    if (PR::kTf32) {
                        const uint32_t h = to_tf32(v);
                        hi[dst[j]] = h;
                        if (PR::kSplit) lo[dst[j]] = __float_as_uint(v - __uint_as_float(h));
                    } else {
                        // BF16 record: halves x, y, z at 8 n + c
                        const int hw = (dst[j] >> 2) * 8 + (dst[j] & 3);
                        const __nv_bfloat16 h = __float2bfloat16_rn(v);
                        reinterpret_cast<__nv_bfloat16 *>(hi)[hw] = h;
                        if (PR::kSplit)
                            reinterpret_cast<__nv_bfloat16 *>(lo)[hw] = __float2bfloat16_rn(v - __bfloat162float(h));
                    }
                }
                if (m.y < m.z) {
                    float *Eu = u + kCOwn * 4;
                    for (int e = ct; e < 128; e += kCConvThreads) Eu[e] = re[(e >> 3) * 12 + oe + (e & 7)];
                }
                fence_async_smem();  // the records are read by the tensor core (async proxy)
            }
            __syncwarp();
            if (lane == 0) {
                if (warp == 2) {
                    meta_conv[cs] = m;
                    meta_u[us] = m;
                }
                mbar_arrive(bar(kCBarRawEmpty + rs));
                mbar_arrive(bar(kCBarConvFull + cs));
                mbar_arrive(bar(kCBarUFull + us));
            }
            if (m.x < 0) break;
        }
    } else {
        // ------------------------------------------------------------ drain
        const int dw = warp & 3;                   // TMEM lane quarter (warps 8-11)
        const int r = dw * 32 + lane, ex = lane & 7, ey = r >> 3;
        float *xch = reinterpret_cast<float *>(smem + kC_OffX);
        uint32_t es = 0, xk = 0, rk = 0;
        float top[3] = {0.0f, 0.0f, 0.0f}, part = 0.0f;
        MfProblem P{};
        int x0 = 0, y0 = 0, z0 = 0, prob = 0;
        bool own = false;
        for (uint32_t k = 0;; k++) {
            const int us = (int)(k % kCNU);
            bool ok = col_wait(bar(kCBarUFull + us), (k / kCNU) & 1u, abort_flag);
            ok = __all_sync(0xffffffffu, ok);
            if (!ok) break;
            const int4 m = meta_u[us];
            if (m.x < 0) break;
            const float *u = reinterpret_cast<const float *>(smem + kC_OffU + us * kCUSlot);
            if (m.y == 0) {
                const MfCol cl = cols[m.x];
                prob = cl.prob;
                P = probs[prob];
                x0 = cl.cx * kCX;
                y0 = cl.cy * kCY;
                z0 = cl.cz * P.col_z;
                own = ex >= 1 && ey >= 1 && x0 + ex - 1 < P.NX && y0 + ey - 1 < P.NY;
                part = 0.0f;
                top[0] = top[1] = top[2] = 0.0f;
            }
            if (m.y < m.z) {
                // element plane s = m.y: its accumulator, scaled by E_e
                const int ts = (int)(es % kCNT);
                ok = col_wait(bar(kCBarTFull + ts), (es / kCNT) & 1u, abort_flag);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) break;
                fence_after();
                float v[24];
                {
                    const uint32_t ta = tmem + ((uint32_t)(dw * 32) << 16) + (uint32_t)ts * kCTCols;
                    tmem_ld24(ta, v);
                    if (PR::kSplit) {
                        float w[24];
                        tmem_ld24(ta + 32, w);
#pragma unroll
                        for (int i = 0; i < 24; i++) v[i] += w[i];
                    }
                }
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar(kCBarTEmpty + ts));
                es++;
                const float e = u[kCOwn * 4 + r];
                // in-plane sums: A = row-ey corners of node (ex, ey), B = row-ey corners of
                // node (ex, ey + 1); [0] bottom corners (dz = 0), [1] top corners (dz = 1)
                float A[2][3], B[2][3];
#pragma unroll
                for (int dz = 0; dz < 2; dz++)
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float a00 = e * v[3 * corner_index(0, 0, dz) + c];
                        const float a10 = e * v[3 * corner_index(1, 0, dz) + c];
                        const float a01 = e * v[3 * corner_index(0, 1, dz) + c];
                        const float a11 = e * v[3 * corner_index(1, 1, dz) + c];
                        A[dz][c] = a00 + __shfl_up_sync(0xffffffffu, a10, 1);
                        B[dz][c] = a01 + __shfl_up_sync(0xffffffffu, a11, 1);
                    }
                // B of the row below: within the warp by a shuffle, across warps through
                // shared memory (the previous warp's last row)
                float Bp[2][3];
#pragma unroll
                for (int dz = 0; dz < 2; dz++)
#pragma unroll
                    for (int c = 0; c < 3; c++) Bp[dz][c] = __shfl_up_sync(0xffffffffu, B[dz][c], 8);
                const int xs2 = (int)(xk & 1u);
                float *xw = xch + xs2 * kCXch;
                if (lane >= 24) {
#pragma unroll
                    for (int dz = 0; dz < 2; dz++)
#pragma unroll
                        for (int c = 0; c < 3; c++) xw[(dw * 8 + ex) * 8 + dz * 3 + c] = B[dz][c];
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(bar(kCBarXch + xs2));
                ok = col_wait(bar(kCBarXch + xs2), (xk >> 1) & 1u, abort_flag);
                ok = __all_sync(0xffffffffu, ok);
                if (!ok) break;
                xk++;
                if (lane < 8 && dw > 0) {
#pragma unroll
                    for (int dz = 0; dz < 2; dz++)
#pragma unroll
                        for (int c = 0; c < 3; c++) Bp[dz][c] = xw[((dw - 1) * 8 + ex) * 8 + dz * 3 + c];
                }
                // node plane m.y = bottom corners of element plane m.y + top corners of m.y - 1
                if (m.y >= 1 && own) {
                    const int gx = x0 + ex - 1, gy = y0 + ey - 1, gz = z0 - 1 + m.y;
                    const int64_t gd = dof_index(P, gx, gy, gz, 0);
                    float4 uv = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    if (MODE == 1) uv = *reinterpret_cast<const float4 *>(u + ((ey - 1) * kCX + ex - 1) * 4);
                    const float un[3] = {uv.x, uv.y, uv.z};
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float acc = (A[0][c] + Bp[0][c]) + top[c];
                        if (MODE == 1) {
                            y[gd + c] = acc;
                            p_new[gd + c] = un[c];
                            part = fmaf(un[c], acc, part);
                        } else if (MODE == 2) {
                            y[gd + c] = (dinv[gd + c] == 0.0f) ? 0.0f : rhs[gd + c] - acc;
                        } else {
                            y[gd + c] = (dinv[gd + c] == 0.0f) ? 0.0f : acc;
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; c++) top[c] = A[1][c] + Bp[1][c];
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(kCBarUEmpty + us));
            if (MODE == 1 && m.y == m.z) {
                // column partial of p.q: FP32 within a warp, FP64 across the four warps
                float w = part;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
                const int rb = (int)(rk & 1u);
                if (lane == 0) {
                    red[rb * 4 + dw] = (double)w;
                    mbar_arrive(bar(kCBarRed + rb));
                }
                if (dw == 0) {
                    ok = col_wait(bar(kCBarRed + rb), (rk >> 1) & 1u, abort_flag);
                    ok = __all_sync(0xffffffffu, ok);
                    if (!ok) break;
                    MfState *st = states + prob;
                    int last = 0;
                    if (lane == 0) {
                        const double sum = ((red[rb * 4] + red[rb * 4 + 1]) + red[rb * 4 + 2]) + red[rb * 4 + 3];
                        col_part[m.x] = sum;
                        __threadfence();
                        const unsigned tk = atomicAdd(&st->cnt_apply, 1u);
                        last = (tk + 1u == (unsigned)P.col_count);
                    }
                    last = __shfl_sync(0xffffffffu, last, 0);
                    if (last) {
                        __threadfence();
                        // eight independent loads in flight per lane, added in column order
                        double s = 0.0;
                        for (int c0 = lane; c0 < P.col_count; c0 += 32 * 8) {
                            double pv[8];
#pragma unroll
                            for (int t = 0; t < 8; t++) {
                                const int c = c0 + 32 * t;
                                pv[t] = c < P.col_count ? __ldcg(col_part + P.col_begin + c) : 0.0;
                            }
#pragma unroll
                            for (int t = 0; t < 8; t++) s += pv[t];
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                        if (lane == 0) {
                            st->cnt_apply = 0;
                            st->pq = s;
                            if (is_bad(s)) { st->status = MG_ENAN; st->done = 1; }
                            else if (!(s > 0.0)) { st->status = MG_EBREAKDOWN; st->done = 1; }
                            else st->alpha = st->rz / s;
                        }
                    }
                }
                rk++;
            }
        }
        if (*abort_flag && lane == 0) atomicOr(err, 2);
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 1) tmem_dealloc(tmem, kCNT * kCTCols);
}

// ------------------------------------------------- factored CUDA-core operator
// y = sum_e E_e P_e^T K0 P_e x in FP32 on the CUDA cores with the factored
// element stiffness (hex8_factored.cuh: 2 x 72 butterfly additions + 45 FMA per
// element instead of 576 FMA), two elements per thread in packed FP32x2
// arithmetic.  A tile owns kFNX x kFNY nodes in x, y and P.fac_z node planes
// in z and streams through its element planes.  Warp w holds element rows 2w
// and 2w+1 of the kFEX x kFEY element plane around the owned nodes (lane = x;
// halo elements are recomputed by the neighbouring tiles).  The node planes
// (input, D^-1 and the per-mode node vectors) and the moduli plane arrive by
// TMA two planes ahead into a four-slot ring.  Per element plane: gather the
// corner values from the two node planes, apply the factored stiffness scaled
// by E_e, then sum the corner results into the owned nodes: along x with a warp
// shuffle (left element + right element), along y inside the thread (rows 2w,
// 2w+1) or through shared memory (row 2w+1 with the next warp's row 2w+2),
// along z through registers (the top corners of plane z-1 + the bottom corners
// of plane z).  Every node's sum has the same fixed order (deterministic and
// independent of the tiling).
constexpr int kFEX = 32, kFEY = 16;                // elements per tile plane
constexpr int kFNX = kFEX - 1, kFNY = kFEY - 1;    // owned nodes per tile plane
constexpr int kFPX = kFEX + 1, kFPY = kFEY + 1;    // tile node plane (with halo)
constexpr int kFThreads = 256;                     // 8 warps x 2 element rows
constexpr int kFMinZ = 1, kFMaxZ = 32;
constexpr int kFRing = 4;                          // 2 planes read, 2 in flight
constexpr int kFBoxX = 104;                        // TMA node box: 104 floats (3 kFPX + alignment) x kFPY rows
constexpr int kFPlaneF = 1792;                     // floats per node plane in the ring (7168 B, 128 B aligned)
constexpr int kFBoxE = 36;                         // TMA moduli box: 36 elements x kFEY rows
constexpr int kFModF = kFBoxE * kFEY;              // 576 floats
constexpr int kFXch = 6 * kFThreads;               // row exchange: 6 floats per thread
static_assert(kFBoxX * kFPY <= kFPlaneF && kFBoxX >= 3 + 3 * kFPX && kFBoxE >= 3 + kFEX, "boxes");
static_assert(kFThreads == 32 * (kFEY / 2) && kFEX == 32, "warp = element row pair, lane = x");
// tensor maps per problem for this kernel: node vectors with the 104 x 17 x 1 box
// and the moduli with the 36 x 16 x 1 box
enum FacMap { kFMapMx = 0, kFMapMd, kFMapMy, kFMapMb, kFMapR, kFMapDinv, kFMapMr, kFMapE, kFacMaps };
// node planes per ring slot: the input, D^-1 and (MODE 2 rhs, MODE 4 r, MODE 5 the iterate)
__host__ __device__ constexpr int fac_planes(int mode) { return mode == 3 ? 2 : 3; }
__host__ __device__ constexpr int fac_slot(int mode) { return fac_planes(mode) * kFPlaneF + kFModF; }
__host__ __device__ constexpr int fac_smem(int mode) { return (kFRing * fac_slot(mode) + 2 * kFXch) * 4 + 128; }
// MODE 3: 77,696 B; MODE 2, 4, 5: 106,368 B: two CTAs per SM

struct FacArgs {
    int in_map, b_map;  // tensor maps (FacMap) of the input and of the third node plane
    float *y;           // MODE 2, 3: output; MODE 4, 5: the new direction
    float *r, *xs;      // MODE 4, 5: Chebyshev residual and iterate
    float c1, c2, inv_theta;
    int x0_zero;        // MODE 5: the iterate starts at 0 (its plane is not loaded)
};

// MODE 2: y = rhs - A x.  MODE 3: y = A x.  (Both 0 where dinv = 0.)
// MODE 4: one Chebyshev step on direction x = d: r -= A d; y = d' = c1 d +
//         c2 D^-1 r; xs += d' (mg_cheb_next_kernel's sequence, fused).
// MODE 5: the first two Chebyshev steps on rhs x = b: d = D^-1 b / theta,
//         xs (+)= d, r = b - A d, y = d' = c1 d + c2 D^-1 r, xs += d'
//         (mg_cheb_first_kernel's and mg_cheb_next_kernel's sequence, fused).
// A TMA wait that exceeds its bound sets bit 4 of *err and ends the block.
template <int MODE>
__global__ void __launch_bounds__(kFThreads, 2) mf_fac_kernel(
    const MfProblem *__restrict__ probs, const MfCol *__restrict__ tiles, int t_lo, int t_hi, int sel,
    const FacK2 K, const CUtensorMap *__restrict__ fmaps, const MfState *__restrict__ states, const FacArgs A,
    int *err) {
    pdl_trigger();
    extern __shared__ __align__(128) float fsm[];
    __shared__ __align__(8) uint64_t bars[kFRing];
    constexpr int NP = fac_planes(MODE);
    // slot k: [input plane | D^-1 plane | third plane (NP = 3) | moduli]
    auto plane_of = [&](int slot, int part) { return fsm + slot * fac_slot(MODE) + part * kFPlaneF; };
    auto mod_of = [&](int slot) { return fsm + slot * fac_slot(MODE) + NP * kFPlaneF; };
    float(*sX)[6][kFThreads] = reinterpret_cast<float(*)[6][kFThreads]>(fsm + kFRing * fac_slot(MODE));
    const int tid = threadIdx.x, tx = tid & 31, w = tid >> 5;
    const uint32_t bar0 = smem_u32(&bars[0]);
    if (tid == 0)
        for (int k = 0; k < kFRing; k++) mbar_init(bar0 + 8 * k, 1);
    // the tile and problem tables are constant: bring the first tile's into the
    // caches while the previous kernel drains, then wait for its results
    if (t_lo + (int)blockIdx.x < t_hi && tid == 0) {
        const MfCol T0 = tiles[t_lo + blockIdx.x];
        asm volatile("prefetch.global.L1 [%0];" ::"l"(probs + T0.prob));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(fmaps + (size_t)T0.prob * kFacMaps));
    }
    pdl_wait();
    __syncthreads();
    uint32_t phase = 0;   // bit k: parity of slot k's next completion
    uint32_t issued = 0;  // bit k: a load into slot k is outstanding (thread 0)
    bool failed = false;
    const bool third = MODE == 2 || MODE == 4 || (MODE == 5 && !A.x0_zero);
    for (int ti = t_lo + blockIdx.x; ti < t_hi && !failed; ti += gridDim.x) {
        const MfCol T = tiles[ti];
        const MfProblem P = probs[T.prob];
        if (states[P.root].done || P.bottom || (sel >= 0 && sel != (P.coarse < 0 ? 1 : 0))) continue;
        const int x0 = T.cx * kFNX, y0 = T.cy * kFNY, z0 = T.cz * P.fac_z;
        const int z1 = min(z0 + P.fac_z, P.NZ);
        const int S = z1 - z0 + 1;  // element planes z0-1 .. z1-1; node planes z0-1 .. z1
        // 16-byte aligned box starts and the offsets of the tile inside the boxes
        const int xs = (3 * (x0 - 1)) & ~3, ox = 3 * (x0 - 1) - xs;
        const int xe = (x0 - 1) & ~3, oe = (x0 - 1) - xe;
        const CUtensorMap *maps = fmaps + (size_t)T.prob * kFacMaps;
        const int64_t plane_stride = (int64_t)P.NY * P.pitch;
        const uint32_t bytes = (uint32_t)(((third ? 3 : 2) * kFBoxX * kFPY + kFModF) * 4);
        // node planes p (nz = z0 - 1 + p) and element plane p's moduli into slot p % kFRing
        auto issue = [&](int p) {
            const int slot = p % kFRing;
            const uint32_t bar = bar0 + 8 * slot;
            fence_async_smem();
            mbar_expect_tx(bar, bytes);
            tma_load_3d(smem_u32(plane_of(slot, 0)), maps + A.in_map, xs, y0 - 1, z0 - 1 + p, bar);
            tma_load_3d(smem_u32(plane_of(slot, 1)), maps + kFMapDinv, xs, y0 - 1, z0 - 1 + p, bar);
            if (third) tma_load_3d(smem_u32(plane_of(slot, 2)), maps + A.b_map, xs, y0 - 1, z0 - 1 + p, bar);
            tma_load_3d(smem_u32(mod_of(slot)), maps + kFMapE, xe, y0 - 1, z0 - 1 + p, bar);
        };
        // every thread waits for slot p's loads; false after the bound
        auto arrive = [&](int p) {
            const int slot = p % kFRing;
            const bool ok = mbar_wait_bounded(bar0 + 8 * slot, (phase >> slot) & 1u);
            phase ^= 1u << slot;
            if (tid == 0) issued &= ~(1u << slot);
            return ok;
        };
        // owned nodes: x = x0 + tx; rows y0 + 2w (row 2w+1 of the tile plane) and
        // y0 + 2w + 1 (row 2w+2, warps 0..6)
        const int gx = x0 + tx, gy1 = y0 + 2 * w, gy2 = gy1 + 1;
        const bool own1 = tx < kFNX && gx < P.NX && gy1 < P.NY;
        const bool own2 = tx < kFNX && w < kFEY / 2 - 1 && gx < P.NX && gy2 < P.NY;
        __syncthreads();  // the previous tile's readers of the ring and the exchange are done
        if (tid == 0) {
            for (int p = 0; p < 3 && p <= S; p++) {
                issue(p);
                issued |= 1u << (p % kFRing);
            }
        }
        bool ok = arrive(0);
        ok = arrive(1) && ok;
        float pt[2][3] = {{0.0f, 0.0f, 0.0f}, {0.0f, 0.0f, 0.0f}};  // top-corner sums of the previous plane
        int64_t g1 = P.dof_off + ((int64_t)(z0 - 1) * P.NY + gy1) * P.pitch + 3 * gx;
        for (int s = 0; s < S; s++) {
            // plane s + 3 into the slot of plane s - 1, whose readers (the element phases
            // of steps s - 2, s - 1 and the node-phase reads of step s - 1) are behind
            // the barrier of step s - 1
            if (tid == 0 && s + 3 <= S) {
                issue(s + 3);
                issued |= 1u << ((s + 3) % kFRing);
            }
            // element phase: corner values of the element pair, packed (A in .x, B in .y)
            float2 v[3][8];
            {
                const float *n0 = plane_of(s % kFRing, 0) + ox, *n1 = plane_of((s + 1) % kFRing, 0) + ox;
                const float *m0 = plane_of(s % kFRing, 1) + ox, *m1 = plane_of((s + 1) % kFRing, 1) + ox;
                float nv[2][3][2][3];  // [bz][row 2w + 0..2][bx][c]
#pragma unroll
                for (int bz = 0; bz < 2; bz++)
#pragma unroll
                    for (int r3 = 0; r3 < 3; r3++)
#pragma unroll
                        for (int bx = 0; bx < 2; bx++) {
                            const int o = (2 * w + r3) * kFBoxX + 3 * (tx + bx);
#pragma unroll
                            for (int c = 0; c < 3; c++) {
                                float val = (bz ? n1 : n0)[o + c];
                                if (MODE == 5) val = (bz ? m1 : m0)[o + c] * val * A.inv_theta;
                                nv[bz][r3][bx][c] = val;
                            }
                        }
#pragma unroll
                for (int b = 0; b < 8; b++) {
                    const int bx = b & 1, by = (b >> 1) & 1, bz = b >> 2;
#pragma unroll
                    for (int c = 0; c < 3; c++) v[c][b] = make_float2(nv[bz][by][bx][c], nv[bz][by + 1][bx][c]);
                }
            }
            const float *Es = mod_of(s % kFRing) + oe + tx;
            const float2 e2 = make_float2(Es[2 * w * kFBoxE], Es[(2 * w + 1) * kFBoxE]);
            hex8_factored_apply2(K, e2, v);  // E = 0 (outside the grid) gives exact zeros
            // along x: node x0 + tx = corner dx = 1 of this lane's element + dx = 0 of the next lane's
            float2 xsum[3][2][2];  // [c][by][bz]
#pragma unroll
            for (int c = 0; c < 3; c++)
#pragma unroll
                for (int by = 0; by < 2; by++)
#pragma unroll
                    for (int bz = 0; bz < 2; bz++) {
                        const float2 lo = v[c][2 * by + 4 * bz], hi = v[c][1 + 2 * by + 4 * bz];
                        float2 nb;
                        nb.x = __shfl_down_sync(0xffffffffu, lo.x, 1);
                        nb.y = __shfl_down_sync(0xffffffffu, lo.y, 1);
                        xsum[c][by][bz] = __fadd2_rn(hi, nb);
                    }
            // along y: row 2w of this warp (element 2w at by = 0) goes to the warp above
            float(*X)[kFThreads] = sX[s & 1];
#pragma unroll
            for (int bz = 0; bz < 2; bz++)
#pragma unroll
                for (int c = 0; c < 3; c++) X[bz * 3 + c][tid] = xsum[c][0][bz].x;
            // node-phase inputs at the owned nodes of node plane s (its slot is refilled
            // in the next step): the input in un, D^-1 in dv, the third plane in bv
            float un[2][3], dv[2][3], bv[2][3];
#pragma unroll
            for (int rr = 0; rr < 2; rr++) {
                const int o = ox + (2 * w + 1 + rr) * kFBoxX + 3 * (tx + 1);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    un[rr][c] = plane_of(s % kFRing, 0)[o + c];
                    dv[rr][c] = plane_of(s % kFRing, 1)[o + c];
                    bv[rr][c] = third ? plane_of(s % kFRing, 2)[o + c] : 0.0f;
                }
            }
            // the next step's top plane (s + 2) has landed
            bool sok = true;
            if (s + 2 <= S) sok = arrive(s + 2);
            if (__syncthreads_or(!(sok && ok))) {
                failed = true;
                if (tid == 0) atomicOr(err, 4);
                break;
            }
            float nn[2][2][3];  // [row][bz][c]; node plane z0 - 1 + s gets its bottom-corner sums now
#pragma unroll
            for (int bz = 0; bz < 2; bz++)
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    nn[0][bz][c] = xsum[c][1][bz].x + xsum[c][0][bz].y;  // element 2w (by = 1) + 2w+1 (by = 0)
                    nn[1][bz][c] = xsum[c][1][bz].y + (w < kFEY / 2 - 1 ? X[bz * 3 + c][tid + 32] : 0.0f);
                }
#pragma unroll
            for (int rr = 0; rr < 2; rr++) {
                const bool own = rr ? own2 : own1;
                if (own && s >= 1) {
                    const int64_t g = g1 + (rr ? P.pitch : 0);
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float a = pt[rr][c] + nn[rr][0][c];
                        if (MODE == 2) {
                            A.y[g + c] = dv[rr][c] == 0.0f ? 0.0f : bv[rr][c] - a;
                        } else if (MODE == 3) {
                            A.y[g + c] = dv[rr][c] == 0.0f ? 0.0f : a;
                        } else if (MODE == 4) {
                            const float rv = bv[rr][c] - (dv[rr][c] == 0.0f ? 0.0f : a);
                            const float dn2 = fmaf(A.c1, un[rr][c], A.c2 * dv[rr][c] * rv);
                            A.r[g + c] = rv;
                            A.y[g + c] = dn2;
                            A.xs[g + c] += dn2;
                        } else {
                            // d = D^-1 b / theta at the node, its iterate, residual and next direction
                            const float dd = dv[rr][c], bb = un[rr][c];
                            const float d0 = dd * bb * A.inv_theta;
                            const float xv = A.x0_zero ? d0 : bv[rr][c] + d0;
                            const float rv = bb - (dd == 0.0f ? 0.0f : a);
                            const float dn2 = fmaf(A.c1, d0, A.c2 * dd * rv);
                            A.r[g + c] = rv;
                            A.y[g + c] = dn2;
                            A.xs[g + c] = xv + dn2;
                        }
                    }
                }
#pragma unroll
                for (int c = 0; c < 3; c++) pt[rr][c] = nn[rr][1][c];
            }
            g1 += plane_stride;
        }
    }
    // after a failed wait, give the outstanding loads a bounded chance to land
    if (failed && tid == 0)
        for (int k = 0; k < kFRing; k++)
            if (issued & (1u << k)) (void)mbar_wait_bounded(bar0 + 8 * k, (phase >> k) & 1u);
    __syncthreads();
}

// ---------------------------------------------------------------- vector phase
// x += alpha p; r -= alpha q (r stays 0 on Dirichlet dofs, D^-1 = 0 there);
// z = D^-1 r; rz, rr -> beta, stop test.  float4 over 16-byte aligned chunks.
// mg = 1: z comes from the multigrid V-cycle; only rr (stop test) is reduced
// here and beta is formed after the V-cycle (mf_dot_rz_kernel).
__global__ void __launch_bounds__(kThreads) mf_update_kernel(
    const MfChunkDesc *__restrict__ chunks, int n_chunks, const MfProblem *__restrict__ probs,
    float *__restrict__ x, float *__restrict__ r, float *__restrict__ z,
    const float *__restrict__ p, const float *__restrict__ q, const float *__restrict__ dinv,
    MfState *states, double *__restrict__ chunk_part, int mg) {
    pdl_enter();
    __shared__ double red_sh[kThreads / 32];
    __shared__ int sh_last;
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x) {
        const MfChunkDesc C = chunks[ci];
        MfState *st = states + C.prob;
        if (st->done) continue;
        const float alpha = (float)st->alpha;
        float rz = 0.0f, rr = 0.0f;
#pragma unroll 4
        for (int64_t i = C.begin + 4 * threadIdx.x; i < C.end; i += 4 * kThreads) {
            const float4 pv = *reinterpret_cast<const float4 *>(p + i);
            const float4 qv = *reinterpret_cast<const float4 *>(q + i);
            const float4 dv = *reinterpret_cast<const float4 *>(dinv + i);
            float4 xv = *reinterpret_cast<const float4 *>(x + i);
            float4 rv = *reinterpret_cast<const float4 *>(r + i);
            xv.x = fmaf(alpha, pv.x, xv.x); xv.y = fmaf(alpha, pv.y, xv.y);
            xv.z = fmaf(alpha, pv.z, xv.z); xv.w = fmaf(alpha, pv.w, xv.w);
            rv.x = dv.x != 0.0f ? fmaf(-alpha, qv.x, rv.x) : 0.0f;
            rv.y = dv.y != 0.0f ? fmaf(-alpha, qv.y, rv.y) : 0.0f;
            rv.z = dv.z != 0.0f ? fmaf(-alpha, qv.z, rv.z) : 0.0f;
            rv.w = dv.w != 0.0f ? fmaf(-alpha, qv.w, rv.w) : 0.0f;
            const float4 zv = make_float4(dv.x * rv.x, dv.y * rv.y, dv.z * rv.z, dv.w * rv.w);
            *reinterpret_cast<float4 *>(x + i) = xv;
            *reinterpret_cast<float4 *>(r + i) = rv;
            if (!mg) *reinterpret_cast<float4 *>(z + i) = zv;
            rz = fmaf(rv.x, zv.x, fmaf(rv.y, zv.y, fmaf(rv.z, zv.z, fmaf(rv.w, zv.w, rz))));
            rr = fmaf(rv.x, rv.x, fmaf(rv.y, rv.y, fmaf(rv.z, rv.z, fmaf(rv.w, rv.w, rr))));
        }
        const double srz = block_sum_f(rz, red_sh);
        const double srr = block_sum_f(rr, red_sh);
        const MfProblem &P = probs[C.prob];
        if (threadIdx.x == 0) {
            chunk_part[ci] = srz;
            chunk_part[n_chunks + ci] = srr;
            __threadfence();
            const unsigned t = atomicAdd(&st->cnt_update, 1u);
            sh_last = (t == (unsigned)P.chunk_count - 1);
        }
        __syncthreads();
        if (sh_last) {
            const double trz = ordered_sum(chunk_part, P.chunk_begin, P.chunk_count);
            const double trr = ordered_sum(chunk_part + n_chunks, P.chunk_begin, P.chunk_count);
            if (threadIdx.x == 0) {
                st->cnt_update = 0;
                st->iter += 1;
                st->total_iter += 1;
                st->rr = trr;
                if (is_bad(trr) || (!mg && is_bad(trz))) { st->status = MG_ENAN; st->done = 1; }
                else {
                    if (!mg) {
                        st->beta = trz / st->rz;
                        st->rz = trz;
                    }
                    if (trr <= st->tol2) st->done = 1;
                    else if (st->iter >= st->maxit) { st->status = MG_ENOCONV; st->done = 1; }
                }
            }
        }
        __syncthreads();
    }
}

// rz = r . z after the V-cycle; init: beta = 0, else beta = rz / rz_old
__global__ void __launch_bounds__(kThreads) mf_dot_rz_kernel(
    const MfChunkDesc *__restrict__ chunks, int n_chunks, const MfProblem *__restrict__ probs,
    const float *__restrict__ r, const float *__restrict__ z, MfState *states,
    double *__restrict__ chunk_part, int init) {
    pdl_enter();
    __shared__ double red_sh[kThreads / 32];
    __shared__ int sh_last;
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x) {
        const MfChunkDesc C = chunks[ci];
        MfState *st = states + C.prob;
        if (st->done) continue;
        float rz = 0.0f;
#pragma unroll 4
        for (int64_t i = C.begin + 4 * threadIdx.x; i < C.end; i += 4 * kThreads) {
            const float4 rv = *reinterpret_cast<const float4 *>(r + i);
            const float4 zv = *reinterpret_cast<const float4 *>(z + i);
            rz = fmaf(rv.x, zv.x, fmaf(rv.y, zv.y, fmaf(rv.z, zv.z, fmaf(rv.w, zv.w, rz))));
        }
        const double srz = block_sum_f(rz, red_sh);
        const MfProblem &P = probs[C.prob];
        if (threadIdx.x == 0) {
            chunk_part[ci] = srz;
            __threadfence();
            const unsigned t = atomicAdd(&st->cnt_update, 1u);
            sh_last = (t == (unsigned)P.chunk_count - 1);
        }
        __syncthreads();
        if (sh_last) {
            const double trz = ordered_sum(chunk_part, P.chunk_begin, P.chunk_count);
            if (threadIdx.x == 0) {
                st->cnt_update = 0;
                if (is_bad(trz) || !(trz > 0.0)) {
                    // a preconditioner that is not positive on r: stop with breakdown
                    st->status = is_bad(trz) ? MG_ENAN : MG_EBREAKDOWN;
                    st->done = 1;
                } else {
                    st->beta = (init || st->first) ? 0.0 : trz / st->rz;
                    st->rz = trz;
                    st->first = 0;
                }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ multigrid kernels
// Chebyshev-Jacobi smoothing (first step): mr = rin; md = D^-1 rin / theta;
// mx = md (x0_zero) or mx + md.  Skips designs whose CG has stopped.
__global__ void __launch_bounds__(kThreads) mg_cheb_first_kernel(
    const MfChunkDesc *__restrict__ chunks, int lo, int hi, const MfProblem *__restrict__ probs,
    const MfState *states, const float *__restrict__ rin, float *__restrict__ mr,
    float *__restrict__ md, float *__restrict__ mx, const float *__restrict__ dinv,
    float inv_theta, int x0_zero, int sel) {
    pdl_enter();
    for (int ci = lo + blockIdx.x; ci < hi; ci += gridDim.x) {
        const MfChunkDesc C = chunks[ci];
        const MfProblem &Q = probs[C.prob];
        if (states[Q.root].done || Q.bottom || (sel >= 0 && sel != (Q.coarse < 0 ? 1 : 0))) continue;
#pragma unroll 4
        for (int64_t i = C.begin + 4 * threadIdx.x; i < C.end; i += 4 * kThreads) {
            const float4 rv = *reinterpret_cast<const float4 *>(rin + i);
            const float4 dv = *reinterpret_cast<const float4 *>(dinv + i);
            const float4 d = make_float4(dv.x * rv.x * inv_theta, dv.y * rv.y * inv_theta,
                                         dv.z * rv.z * inv_theta, dv.w * rv.w * inv_theta);
            float4 xv = x0_zero ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4 *>(mx + i);
            xv.x += d.x; xv.y += d.y; xv.z += d.z; xv.w += d.w;
            if (mr != rin) *reinterpret_cast<float4 *>(mr + i) = rv;
            *reinterpret_cast<float4 *>(md + i) = d;
            *reinterpret_cast<float4 *>(mx + i) = xv;
        }
    }
}

// Chebyshev step: mr -= A md (= my); md = c1 md + c2 D^-1 mr; mx += md
__global__ void __launch_bounds__(kThreads) mg_cheb_next_kernel(
    const MfChunkDesc *__restrict__ chunks, int lo, int hi, const MfProblem *__restrict__ probs,
    const MfState *states, const float *__restrict__ my, float *__restrict__ mr,
    float *__restrict__ md, float *__restrict__ mx, const float *__restrict__ dinv, float c1,
    float c2, int sel) {
    pdl_enter();
    for (int ci = lo + blockIdx.x; ci < hi; ci += gridDim.x) {
        const MfChunkDesc C = chunks[ci];
        const MfProblem &Q = probs[C.prob];
        if (states[Q.root].done || Q.bottom || (sel >= 0 && sel != (Q.coarse < 0 ? 1 : 0))) continue;
#pragma unroll 4
        for (int64_t i = C.begin + 4 * threadIdx.x; i < C.end; i += 4 * kThreads) {
            const float4 yv = *reinterpret_cast<const float4 *>(my + i);
            const float4 dv = *reinterpret_cast<const float4 *>(dinv + i);
            float4 rv = *reinterpret_cast<const float4 *>(mr + i);
            float4 d = *reinterpret_cast<const float4 *>(md + i);
            float4 xv = *reinterpret_cast<const float4 *>(mx + i);
            rv.x -= yv.x; rv.y -= yv.y; rv.z -= yv.z; rv.w -= yv.w;
            d.x = fmaf(c1, d.x, c2 * dv.x * rv.x); d.y = fmaf(c1, d.y, c2 * dv.y * rv.y);
            d.z = fmaf(c1, d.z, c2 * dv.z * rv.z); d.w = fmaf(c1, d.w, c2 * dv.w * rv.w);
            xv.x += d.x; xv.y += d.y; xv.z += d.z; xv.w += d.w;
            *reinterpret_cast<float4 *>(mr + i) = rv;
            *reinterpret_cast<float4 *>(md + i) = d;
            *reinterpret_cast<float4 *>(mx + i) = xv;
        }
    }
}

// restriction (transpose of trilinear interpolation) into the coarse problems
// plo..phi-1: mb_c[I] = sum_d w(d) my_f[2I + d], d in {-1,0,1}^3, w = prod (1 - |d|/2)
__global__ void __launch_bounds__(256) mg_restrict_kernel(const MfProblem *__restrict__ probs, int plo,
                                                          const MfState *states, const float *__restrict__ my,
                                                          float *__restrict__ mb, const float *__restrict__ dinv) {
    pdl_enter();
    const MfProblem C = probs[plo + blockIdx.y];
    if (states[C.root].done) return;
    const MfProblem F = probs[C.fine];
    if (F.bottom) return;  // inside a bottom chain: restricted by the bottom kernel
    // one coarse node (3 dofs) per thread: its 27 fine neighbours' loads are all
    // issued before the sums (independent, predicated on the grid bounds)
    const int nn = C.NX * C.NY * C.NZ;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += gridDim.x * blockDim.x) {
        const int I = n % C.NX, JK = n / C.NX, J = JK % C.NY, K = JK / C.NY;
        const int64_t o = C.dof_off + ((int64_t)K * C.NY + J) * C.pitch + 3 * I;
        float v[27][3];
#pragma unroll
        for (int q = 0; q < 27; q++) {
            const int dx = q % 3 - 1, dy = (q / 3) % 3 - 1, dz = q / 9 - 1;
            const int ii = 2 * I + dx, j = 2 * J + dy, k = 2 * K + dz;
            const bool in = ii >= 0 && ii < F.NX && j >= 0 && j < F.NY && k >= 0 && k < F.NZ;
            const float *src = my + F.dof_off + (in ? ((int64_t)k * F.NY + j) * F.pitch + 3 * ii : 0);
#pragma unroll
            for (int c = 0; c < 3; c++) v[q][c] = in ? src[c] : 0.0f;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            // the order of the sums: dz outermost, then dy, then dx (as the transpose of prolongation)
            float out = 0.0f;
#pragma unroll
            for (int q = 0; q < 27; q++) {
                const int dx = q % 3 - 1, dy = (q / 3) % 3 - 1, dz = q / 9 - 1;
                const float w = (dz ? 0.5f : 1.0f) * (dy ? 0.5f : 1.0f) * (dx ? 0.5f : 1.0f);
                out = fmaf(w, v[q][c], out);
            }
            mb[o + c] = dinv[o + c] != 0.0f ? out : 0.0f;
        }
    }
}

// prolongation (trilinear) from the coarse levels into the fine problems
// plo..phi-1: mx_f[i] += sum_I w mx_c[I] (skips Dirichlet dofs and padding)
__global__ void __launch_bounds__(256) mg_prolong_kernel(const MfProblem *__restrict__ probs, int plo,
                                                         const MfState *states, float *__restrict__ mx,
                                                         const float *__restrict__ dinv) {
    pdl_enter();
    const MfProblem F = probs[plo + blockIdx.y];
    if (F.coarse < 0 || F.bottom || states[F.root].done) return;  // nothing to add here
    const MfProblem C = probs[F.coarse];
    // one fine node (3 dofs) per thread; its 1, 2, 4 or 8 coarse parents' loads are
    // issued together (the unused ones predicated off)
    const int nn = F.NX * F.NY * F.NZ;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nn; n += gridDim.x * blockDim.x) {
        const int ii = n % F.NX, jk = n / F.NX, j = jk % F.NY, k = jk / F.NY;
        const int64_t o = F.dof_off + ((int64_t)k * F.NY + j) * F.pitch + 3 * ii;
        const float wx = (ii & 1) ? 0.5f : 1.0f, wy = (j & 1) ? 0.5f : 1.0f, wz = (k & 1) ? 0.5f : 1.0f;
        const float w = wx * wy * wz;
        float v[8][3];
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int a = q >> 2, bb = (q >> 1) & 1, cc = q & 1;
            const bool use = (a == 0 || (k & 1)) && (bb == 0 || (j & 1)) && (cc == 0 || (ii & 1));
            const int I = (ii + cc) >> 1, J = (j + bb) >> 1, K = (k + a) >> 1;
            const float *src = mx + C.dof_off + (use ? ((int64_t)K * C.NY + J) * C.pitch + 3 * I : 0);
#pragma unroll
            for (int c = 0; c < 3; c++) v[q][c] = use ? src[c] : 0.0f;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) {
            if (dinv[o + c] == 0.0f) continue;
            float acc = 0.0f;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int a = q >> 2, bb = (q >> 1) & 1, cc = q & 1;
                const bool use = (a == 0 || (k & 1)) && (bb == 0 || (j & 1)) && (cc == 0 || (ii & 1));
                if (use) acc = fmaf(w, v[q][c], acc);
            }
            mx[o + c] += acc;
        }
    }
}

// coarse moduli: E_c = 2 mean(E of the 8 children); the factor 2 is the
// element-size scaling of the 3D stiffness (K(2h) = 2 K(h)), so every level
// uses the fine-grid reference stiffness K0
__global__ void mg_coarsen_kernel(const MfProblem *__restrict__ probs, int plo,
                                  float *__restrict__ E32) {
    const MfProblem C = probs[plo + blockIdx.y];
    const MfProblem F = probs[C.fine];
    const int64_t ne = (int64_t)C.nx * C.ny * C.nz;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int ex = (int)(e % C.nx), ey = (int)((e / C.nx) % C.ny), ez = (int)(e / ((int64_t)C.nx * C.ny));
        float s = 0.0f;
        for (int dz = 0; dz < 2; dz++)
            for (int dy = 0; dy < 2; dy++)
                for (int dx = 0; dx < 2; dx++)
                    s += E32[F.elem_off + ((int64_t)(2 * ez + dz) * F.ny + 2 * ey + dy) * F.pitch_e + 2 * ex + dx];
        E32[C.elem_off + ((int64_t)ez * C.ny + ey) * C.pitch_e + ex] = 0.25f * s;
    }
}

// ------------------------------------------------------ bottom V-cycle (one CTA)
// The small coarse levels of a design (from its chain head down to its
// coarsest grid) are solved by one CTA per chain, entirely in shared memory,
// in FP32 on the CUDA cores: the same Chebyshev-Jacobi smoothers, residuals,
// restriction and prolongation as the level-by-level launches above, without
// one launch per level operation.  Per level the shared memory holds x, b, r,
// d, y, D^-1 (per dof, compact node-interleaved order) and E (per element).
constexpr int kBottomThreads = 512;
constexpr int kBottomSmemMax = 200 * 1024;  // per chain: 576 + sum over levels (18 NN + ne) floats
constexpr int kBottomMaxHeadNodes = 2 * kBottomThreads;

struct BottomLevel {
    int NX, NY, NZ, nx, ny, nz;
    float *x, *b, *r, *d, *y, *dinv, *E;
};

// y = A in on level L (0 on Dirichlet dofs; `in` is 0 there): node-centric
// gather over the node's elements in a fixed order.  Levels of at most
// kBottomLaneNodes nodes use eight lanes per node instead (lane d = dx + 2 dy +
// 4 dz forms the node's rows of element node - d; the partial sums meet in a
// fixed xor butterfly), which shortens the dependent chain per pass eightfold.
constexpr int kBottomLaneNodes = kBottomThreads / 2;
__device__ void bottom_apply(const BottomLevel &L, const float *sK, const float *in, float *out) {
    const int nn = L.NX * L.NY * L.NZ;
    if (nn <= kBottomLaneNodes) {
        const int corner = threadIdx.x & 7;
        const int dx = corner & 1, dy = (corner >> 1) & 1, dz = corner >> 2;
        // this corner's 3 x 24 rows of K0 regrouped per neighbour corner bc (9 values in
        // 12); corner blocks 100 floats apart, so the eight corners of a node read
        // disjoint banks
        const float4 *Kt = reinterpret_cast<const float4 *>(sK + 576 + 100 * corner_index(dx, dy, dz));
        for (int base = 0; base < nn; base += kBottomThreads / 8) {
            const int n = base + (threadIdx.x >> 3);
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
            if (n < nn) {
                const int i = n % L.NX, j = (n / L.NX) % L.NY, k = n / (L.NX * L.NY);
                const int ex = i - dx, ey = j - dy, ez = k - dz;
                if (ex >= 0 && ey >= 0 && ez >= 0 && ex < L.nx && ey < L.ny && ez < L.nz) {
                    const float e = L.E[ex + L.nx * (ey + L.ny * ez)];
                    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
#pragma unroll
                    for (int bc = 0; bc < 8; bc++) {
                        int bx, by, bz;
                        corner_bits(bc, bx, by, bz);
                        const float *u = in + 3 * ((ex + bx) + L.NX * ((ey + by) + L.NY * (ez + bz)));
                        const float u0 = u[0], u1 = u[1], u2 = u[2];
                        const float4 k0 = Kt[3 * bc], k1 = Kt[3 * bc + 1], k2 = Kt[3 * bc + 2];
                        s0 = fmaf(k0.z, u2, fmaf(k0.y, u1, fmaf(k0.x, u0, s0)));
                        s1 = fmaf(k1.y, u2, fmaf(k1.x, u1, fmaf(k0.w, u0, s1)));
                        s2 = fmaf(k2.x, u2, fmaf(k1.w, u1, fmaf(k1.z, u0, s2)));
                    }
                    a0 = e * s0;
                    a1 = e * s1;
                    a2 = e * s2;
                }
            }
#pragma unroll
            for (int off = 1; off < 8; off <<= 1) {
                a0 += __shfl_xor_sync(0xffffffffu, a0, off);
                a1 += __shfl_xor_sync(0xffffffffu, a1, off);
                a2 += __shfl_xor_sync(0xffffffffu, a2, off);
            }
            if (n < nn && corner < 3) {
                const float a = corner == 0 ? a0 : (corner == 1 ? a1 : a2);
                out[3 * n + corner] = L.dinv[3 * n + corner] == 0.0f ? 0.0f : a;
            }
        }
        return;
    }
    for (int n = threadIdx.x; n < nn; n += kBottomThreads) {
        const int i = n % L.NX, j = (n / L.NX) % L.NY, k = n / (L.NX * L.NY);
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
        for (int dz = 0; dz < 2; dz++)
            for (int dy = 0; dy < 2; dy++)
                for (int dx = 0; dx < 2; dx++) {
                    const int ex = i - dx, ey = j - dy, ez = k - dz;
                    if (ex < 0 || ey < 0 || ez < 0 || ex >= L.nx || ey >= L.ny || ez >= L.nz) continue;
                    const float e = L.E[ex + L.nx * (ey + L.ny * ez)];
                    const float *K = sK + 3 * corner_index(dx, dy, dz) * 24;
                    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
#pragma unroll
                    for (int bc = 0; bc < 8; bc++) {
                        int bx, by, bz;
                        corner_bits(bc, bx, by, bz);
                        const float *u = in + 3 * ((ex + bx) + L.NX * ((ey + by) + L.NY * (ez + bz)));
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            s0 = fmaf(K[3 * bc + c], u[c], s0);
                            s1 = fmaf(K[24 + 3 * bc + c], u[c], s1);
                            s2 = fmaf(K[48 + 3 * bc + c], u[c], s2);
                        }
                    }
                    a0 = fmaf(e, s0, a0);
                    a1 = fmaf(e, s1, a1);
                    a2 = fmaf(e, s2, a2);
                }
        out[3 * n] = L.dinv[3 * n] == 0.0f ? 0.0f : a0;
        out[3 * n + 1] = L.dinv[3 * n + 1] == 0.0f ? 0.0f : a1;
        out[3 * n + 2] = L.dinv[3 * n + 2] == 0.0f ? 0.0f : a2;
    }
}

// x (+)= Chebyshev-Jacobi smoothing of degree deg for rhs rin (r, d, y scratch)
__device__ void bottom_smooth(const BottomLevel &L, const float *sK, const float *rin, bool x0_zero, int deg,
                              float inv_theta, const float *c1, const float *c2) {
    const int nd = 3 * L.NX * L.NY * L.NZ;
    for (int q = threadIdx.x; q < nd; q += kBottomThreads) {
        const float rv = rin[q], dv = L.dinv[q] * rv * inv_theta;
        L.r[q] = rv;
        L.d[q] = dv;
        L.x[q] = x0_zero ? dv : L.x[q] + dv;
    }
    __syncthreads();
    for (int k = 1; k < deg; k++) {
        bottom_apply(L, sK, L.d, L.y);
        __syncthreads();
        for (int q = threadIdx.x; q < nd; q += kBottomThreads) {
            const float rv = L.r[q] - L.y[q];
            const float dv = fmaf(c1[k], L.d[q], c2[k] * L.dinv[q] * rv);
            L.r[q] = rv;
            L.d[q] = dv;
            L.x[q] += dv;
        }
        __syncthreads();
    }
}

// r = b - A x  (0 on Dirichlet dofs)
__device__ void bottom_residual(const BottomLevel &L, const float *sK) {
    bottom_apply(L, sK, L.x, L.y);
    __syncthreads();
    const int nd = 3 * L.NX * L.NY * L.NZ;
    for (int q = threadIdx.x; q < nd; q += kBottomThreads) L.r[q] = L.dinv[q] == 0.0f ? 0.0f : L.b[q] - L.y[q];
    __syncthreads();
}

// Direct coarse solve: the coarsest grid of a bottom chain, when it has at most
// kCoarseDirectMax dofs, is solved exactly with the inverse of its assembled
// operator (FP32, formed on the device by mg_coarse_inverse_kernel) instead of a
// Chebyshev smoother of degree cdeg: one matrix-vector product instead of cdeg - 1
// operator applications, each a CTA-wide barrier round.  The operator is assembled from
// the level's moduli and K0 like the level operators (Dirichlet dofs: identity
// rows and zero columns), so the inverse is symmetric and the V-cycle stays a
// fixed symmetric preconditioner.
constexpr int kCoarseDirectMax = 144;

struct BottomCheb {
    float inv_theta_s, inv_theta_c;
    float c1s[32], c2s[32], c1c[32], c2c[32];
};

__global__ void __launch_bounds__(kBottomThreads, 1) mg_bottom_kernel(
    const MfProblem *__restrict__ probs, const int *__restrict__ heads, const MfState *states,
    const float *__restrict__ E32, const float *__restrict__ dinv_g, const float *__restrict__ mb,
    float *__restrict__ mx, const double *__restrict__ K0, BottomCheb cc, int sdeg, int cdeg,
    const int64_t *__restrict__ coarse_off, const float *__restrict__ coarse_inv,
    const int *__restrict__ coarse_ok) {
    pdl_enter();
    extern __shared__ __align__(16) float sbm[];
    const int head = heads[blockIdx.x];
    const MfProblem H = probs[head];
    if (states[H.root].done) return;
    float *sK = sbm;  // 576, then the regrouped copy for the eight-lane apply (8 x 100)
    for (int i = threadIdx.x; i < 576; i += kBottomThreads) sK[i] = (float)K0[i];
    for (int i = threadIdx.x; i < 800; i += kBottomThreads) {
        const int a = i / 100, t = i % 100, bc = t / 12, q = t % 12, r = q / 3, c = q % 3;
        sbm[576 + i] = (t < 96 && q < 9) ? (float)K0[(3 * a + r) * 24 + 3 * bc + c] : 0.0f;
    }
    // carve the levels of the chain
    BottomLevel Lv[kBottomMaxLevels];
    int pl[kBottomMaxLevels];
    int m = 0;
    float *p = sbm + 576 + 800;
    for (int q = head; q >= 0 && m < kBottomMaxLevels; q = probs[q].coarse) {
        const MfProblem P = probs[q];
        BottomLevel &L = Lv[m];
        L.NX = P.NX; L.NY = P.NY; L.NZ = P.NZ;
        L.nx = P.nx; L.ny = P.ny; L.nz = P.nz;
        const int nd = 3 * P.NX * P.NY * P.NZ, ne = P.nx * P.ny * P.nz;
        L.x = p; p += nd;
        L.b = p; p += nd;
        L.r = p; p += nd;
        L.d = p; p += nd;
        L.y = p; p += nd;
        L.dinv = p; p += nd;
        L.E = p; p += ne;
        pl[m] = q;
        m++;
    }
    // the coarsest grid's inverse (direct solve), fetched with the level tables
    const int64_t inv_off = coarse_ok[blockIdx.x] ? coarse_off[blockIdx.x] : -1;
    float *sInv = p;
    if (inv_off >= 0) {
        const BottomLevel &Lc = Lv[m - 1];
        const int ndc = 3 * Lc.NX * Lc.NY * Lc.NZ;
        for (int i = threadIdx.x; i < ndc * ndc; i += kBottomThreads) sInv[i] = coarse_inv[inv_off + i];
    }
    // load E, D^-1 (and the rhs of the head) from the padded global layout
    for (int l = 0; l < m; l++) {
        const MfProblem P = probs[pl[l]];
        BottomLevel &L = Lv[l];
        const int ne = P.nx * P.ny * P.nz, nn = P.NX * P.NY * P.NZ;
        for (int e = threadIdx.x; e < ne; e += kBottomThreads) {
            const int ex = e % P.nx, ey = (e / P.nx) % P.ny, ez = e / (P.nx * P.ny);
            L.E[e] = E32[P.elem_off + ((int64_t)ez * P.ny + ey) * P.pitch_e + ex];
        }
        for (int q = threadIdx.x; q < 3 * nn; q += kBottomThreads) {
            const int n = q / 3, c = q - 3 * n;
            const int i = n % P.NX, j = (n / P.NX) % P.NY, k = n / (P.NX * P.NY);
            const int64_t g = dof_index(P, i, j, k, c);
            L.dinv[q] = dinv_g[g];
            if (l == 0) L.b[q] = L.dinv[q] == 0.0f ? 0.0f : mb[g];
        }
    }
    __syncthreads();
    // down: smooth, residual, restrict
    for (int l = 0; l < m - 1; l++) {
        bottom_smooth(Lv[l], sK, Lv[l].b, true, sdeg, cc.inv_theta_s, cc.c1s, cc.c2s);
        bottom_residual(Lv[l], sK);
        const BottomLevel &F = Lv[l], &C = Lv[l + 1];
        const int ncd = 3 * C.NX * C.NY * C.NZ;
        for (int q = threadIdx.x; q < ncd; q += kBottomThreads) {
            const int n = q / 3, c = q - 3 * n;
            const int I = n % C.NX, J = (n / C.NX) % C.NY, K = n / (C.NX * C.NY);
            float out = 0.0f;
            if (C.dinv[q] != 0.0f)
                for (int dz = -1; dz <= 1; dz++) {
                    const int kk = 2 * K + dz;
                    if (kk < 0 || kk >= F.NZ) continue;
                    for (int dy = -1; dy <= 1; dy++) {
                        const int jj = 2 * J + dy;
                        if (jj < 0 || jj >= F.NY) continue;
                        for (int dx = -1; dx <= 1; dx++) {
                            const int ii = 2 * I + dx;
                            if (ii < 0 || ii >= F.NX) continue;
                            const float w = (dx ? 0.5f : 1.0f) * (dy ? 0.5f : 1.0f) * (dz ? 0.5f : 1.0f);
                            out = fmaf(w, F.r[3 * (ii + F.NX * (jj + F.NY * kk)) + c], out);
                        }
                    }
                }
            C.b[q] = out;
        }
        __syncthreads();
    }
    // coarsest grid of the chain: exact solve with the stored inverse, or smoothing
    {
        const BottomLevel &L = Lv[m - 1];
        if (inv_off >= 0) {
            // four lanes per row, partial sums met by two shuffles (fixed order)
            const int nd = 3 * L.NX * L.NY * L.NZ, part = threadIdx.x & 3;
            for (int q0 = 0; q0 < nd; q0 += kBottomThreads / 4) {
                const int q = q0 + (threadIdx.x >> 2);
                float sacc = 0.0f;
                if (q < nd)
                    for (int r = part; r < nd; r += 4) sacc = fmaf(sInv[q * nd + r], L.b[r], sacc);
                sacc += __shfl_xor_sync(0xffffffffu, sacc, 1);
                sacc += __shfl_xor_sync(0xffffffffu, sacc, 2);
                if (q < nd && part == 0) L.x[q] = L.dinv[q] == 0.0f ? 0.0f : sacc;
            }
            __syncthreads();
        } else {
            bottom_smooth(Lv[m - 1], sK, Lv[m - 1].b, true, cdeg, cc.inv_theta_c, cc.c1c, cc.c2c);
        }
    }
    // up: prolong, residual, post-smooth
    for (int l = m - 2; l >= 0; l--) {
        const BottomLevel &F = Lv[l], &C = Lv[l + 1];
        const int nfd = 3 * F.NX * F.NY * F.NZ;
        for (int q = threadIdx.x; q < nfd; q += kBottomThreads) {
            if (F.dinv[q] == 0.0f) continue;
            const int n = q / 3, c = q - 3 * n;
            const int ii = n % F.NX, jj = (n / F.NX) % F.NY, kk = n / (F.NX * F.NY);
            const int Is[2] = {ii >> 1, (ii + 1) >> 1}, Js[2] = {jj >> 1, (jj + 1) >> 1}, Ks[2] = {kk >> 1, (kk + 1) >> 1};
            const float w = ((ii & 1) ? 0.5f : 1.0f) * ((jj & 1) ? 0.5f : 1.0f) * ((kk & 1) ? 0.5f : 1.0f);
            float acc = 0.0f;
            for (int a = 0; a < ((kk & 1) ? 2 : 1); a++)
                for (int bb = 0; bb < ((jj & 1) ? 2 : 1); bb++)
                    for (int cc2 = 0; cc2 < ((ii & 1) ? 2 : 1); cc2++)
                        acc = fmaf(w, C.x[3 * (Is[cc2] + C.NX * (Js[bb] + C.NY * Ks[a])) + c], acc);
            F.x[q] += acc;
        }
        __syncthreads();
        bottom_residual(Lv[l], sK);
        // post-smoothing on the residual: x += S(r) (the smoother starts from r in place)
        bottom_smooth(Lv[l], sK, Lv[l].r, false, sdeg, cc.inv_theta_s, cc.c1s, cc.c2s);
    }
    // the head's correction back to the padded global layout
    {
        const MfProblem P = probs[head];
        const int nn = P.NX * P.NY * P.NZ;
        for (int q = threadIdx.x; q < 3 * nn; q += kBottomThreads) {
            const int n = q / 3, c = q - 3 * n;
            const int i = n % P.NX, j = (n / P.NX) % P.NY, k = n / (P.NX * P.NY);
            mx[dof_index(P, i, j, k, c)] = Lv[0].x[q];
        }
    }
}

// FP32 inverse of a chain's coarsest-grid operator (the direct coarse solve), one
// CTA per chain, formed whenever the chain's moduli change.  The operator is
// assembled from K0 and the level's moduli (one thread per row, the node's
// elements in a fixed order; Dirichlet rows and columns replaced by the identity;
// the upper triangle taken for both halves), padded to kCoarseDirectMax with the
// identity and inverted in place by the symmetric sweep operator (Goodnight,
// "A tutorial on the SWEEP operator", 1979): sweeping pivot k maps
// a_ij -> a_ij - a_ik a_kj / a_kk (i, j != k), a_ik -> a_ik / a_kk and
// a_kk -> -1 / a_kk; sweeping every pivot leaves -A^-1.  Each thread keeps a 6 x 6
// tile in registers and forms a_ik a_kj as one product, so the tiles stay bitwise
// symmetric and the stored inverse is exactly symmetric (the V-cycle stays a
// fixed symmetric preconditioner).  No pivoting: the pivots of a symmetric
// positive definite matrix are positive.  A pivot that is not (a singular or
// indefinite coarse operator) clears coarse_ok and the bottom kernel smooths that
// chain's coarsest grid instead.
constexpr int kCoarseTile = 6;
constexpr int kCoarseTiles = kCoarseDirectMax / kCoarseTile;
constexpr int kCoarseInvThreads = kCoarseTiles * kCoarseTiles;
constexpr int kCoarseMaxElems = 64;  // nodes <= kCoarseDirectMax / 3 = 48, so elements < 48
constexpr int kCoarseInvSmem =
    (kCoarseDirectMax * kCoarseDirectMax + 576 + kCoarseMaxElems + 3 * kCoarseDirectMax) * 4;
static_assert(kCoarseDirectMax % kCoarseTile == 0, "the sweep tiles cover the padded operator");

__global__ void __launch_bounds__(kCoarseInvThreads, 1) mg_coarse_inverse_kernel(
    const MfProblem *__restrict__ probs, const int *__restrict__ heads, const int *__restrict__ list,
    const float *__restrict__ E32, const float *__restrict__ dinv, const double *__restrict__ K0,
    const int64_t *__restrict__ coarse_off, float *__restrict__ coarse_inv, int *__restrict__ coarse_ok) {
    constexpr int NP = kCoarseDirectMax, T = kCoarseTile;
    extern __shared__ __align__(16) float sci[];
    float *sA = sci;              // NP x NP assembled operator
    float *sK = sA + NP * NP;     // K0 (576)
    float *sE = sK + 576;         // the level's moduli
    float *sv = sE + kCoarseMaxElems;  // pivot rows, double-buffered (2 x NP)
    int *sfix = reinterpret_cast<int *>(sv + 2 * NP);
    __shared__ float s_rcp[2];         // 1 / pivot of each buffered row, formed once by its writer
    const int h = list[blockIdx.x];
    const int64_t off = coarse_off[h];
    if (off < 0) return;
    int c = heads[h];
    while (probs[c].coarse >= 0) c = probs[c].coarse;
    const MfProblem C = probs[c];
    const int nd = 3 * C.NX * C.NY * C.NZ, ne = C.nx * C.ny * C.nz;
    if (nd > NP || ne > kCoarseMaxElems) {  // not a direct chain (the host never lists one)
        if (threadIdx.x == 0) coarse_ok[h] = 0;
        return;
    }
    const int tid = threadIdx.x;
    for (int i = tid; i < 576; i += kCoarseInvThreads) sK[i] = (float)K0[i];
    for (int e = tid; e < ne; e += kCoarseInvThreads) {
        const int ex = e % C.nx, ey = (e / C.nx) % C.ny, ez = e / (C.nx * C.ny);
        sE[e] = E32[C.elem_off + ((int64_t)ez * C.ny + ey) * C.pitch_e + ex];
    }
    for (int q = tid; q < nd; q += kCoarseInvThreads) {
        const int n = q / 3, cq = q - 3 * n;
        const int i = n % C.NX, j = (n / C.NX) % C.NY, k = n / (C.NX * C.NY);
        sfix[q] = dinv[dof_index(C, i, j, k, cq)] == 0.0f;
    }
    __syncthreads();
    for (int q = tid; q < nd; q += kCoarseInvThreads) {
        float *row = sA + q * NP;
        for (int r = 0; r < NP; r++) row[r] = 0.0f;
        const int n = q / 3, cq = q - 3 * n;
        const int i = n % C.NX, jj = (n / C.NX) % C.NY, k = n / (C.NX * C.NY);
        for (int a = 0; a < 8; a++) {
            int dx, dy, dz;
            corner_bits(a, dx, dy, dz);
            const int ex = i - dx, ey = jj - dy, ez = k - dz;
            if (ex < 0 || ey < 0 || ez < 0 || ex >= C.nx || ey >= C.ny || ez >= C.nz) continue;
            const float e = sE[ex + C.nx * (ey + C.ny * ez)];
            for (int bc = 0; bc < 8; bc++) {
                int bx, by, bz;
                corner_bits(bc, bx, by, bz);
                const int m = (ex + bx) + C.NX * ((ey + by) + C.NY * (ez + bz));
                for (int cb = 0; cb < 3; cb++)
                    row[3 * m + cb] = fmaf(e, sK[(3 * a + cq) * 24 + 3 * bc + cb], row[3 * m + cb]);
            }
        }
    }
    __syncthreads();
    const int ti = tid / kCoarseTiles, tj = tid - ti * kCoarseTiles;
    const int i0 = ti * T, j0 = tj * T;
    float a[T][T];
#pragma unroll
    for (int r = 0; r < T; r++)
#pragma unroll
        for (int cc = 0; cc < T; cc++) {
            const int i = i0 + r, j = j0 + cc;
            float v = i == j ? 1.0f : 0.0f;
            if (i < nd && j < nd && !sfix[i] && !sfix[j]) v = i <= j ? sA[i * NP + j] : sA[j * NP + i];
            a[r][cc] = v;
        }
    if (ti == 0)
#pragma unroll
        for (int cc = 0; cc < T; cc++) sv[j0 + cc] = a[0][cc];
    if (tid == 0) s_rcp[0] = 1.0f / a[0][0];
    __syncthreads();
    int ok = 1, cur = 0;
    for (int k = 0; k < nd; k++) {
        const float *v = sv + cur * NP;
        const float d = v[k];  // the same value in every thread: the exit below is uniform
        if (!(d > 0.0f) || !isfinite(d)) {
            ok = 0;
            break;
        }
        const float p = s_rcp[cur];
        float vi[T], vj[T];
#pragma unroll
        for (int r = 0; r < T; r++) {
            vi[r] = v[i0 + r];
            vj[r] = v[j0 + r];
        }
#pragma unroll
        for (int r = 0; r < T; r++)
#pragma unroll
            for (int cc = 0; cc < T; cc++) a[r][cc] = fmaf(-(vi[r] * vj[cc]), p, a[r][cc]);
        const int kr = k - i0, kc = k - j0;
        // row and column k: a_kj = v_j / d, a_ik = v_i / d, a_kk = -1 / d
        if ((unsigned)kr < (unsigned)T) {
#pragma unroll
            for (int r = 0; r < T; r++)
                if (r == kr)
#pragma unroll
                    for (int cc = 0; cc < T; cc++) a[r][cc] = cc == kc ? -p : vj[cc] * p;
        }
        if ((unsigned)kc < (unsigned)T) {
#pragma unroll
            for (int cc = 0; cc < T; cc++)
                if (cc == kc)
#pragma unroll
                    for (int r = 0; r < T; r++)
                        if (r != kr) a[r][cc] = vi[r] * p;
        }
        const int nr = k + 1 - i0;  // the next pivot row (and its reciprocal pivot)
        if ((unsigned)nr < (unsigned)T) {
            float *vn = sv + (cur ^ 1) * NP;
            const int nc = k + 1 - j0;
#pragma unroll
            for (int r = 0; r < T; r++)
                if (r == nr)
#pragma unroll
                    for (int cc = 0; cc < T; cc++) {
                        vn[j0 + cc] = a[r][cc];
                        if (cc == nc) s_rcp[cur ^ 1] = 1.0f / a[r][cc];
                    }
        }
        __syncthreads();
        cur ^= 1;
    }
    if (tid == 0) coarse_ok[h] = ok;
    if (!ok) return;
    float *out = coarse_inv + off;
#pragma unroll
    for (int r = 0; r < T; r++)
#pragma unroll
        for (int cc = 0; cc < T; cc++) {
            const int i = i0 + r, j = j0 + cc;
            if (i < nd && j < nd) out[i * nd + j] = -a[r][cc];
        }
}

// ------------------------------------------------- bottom V-cycle on a cluster
// The same bottom V-cycle as mg_bottom_kernel, spread over a thread-block
// cluster of up to 16 CTAs (one cluster per chain) so that a single design's
// chain can start at a larger level.  CTA r owns the nodes [r chunk, (r + 1) chunk)
// of every level of the chain and keeps their x, b, r, d, y in its shared memory
// (with D^-1 and the moduli of whole levels); a phase reads other CTAs' nodes
// through distributed shared memory (mapa + ld.shared::cluster) and a cluster
// barrier (release / acquire) separates the phases.  Global memory is touched only
// at the start (rhs, tables) and at the end (the head's correction).  Every dof is
// computed by one thread in a fixed order whatever the cluster size, so the result
// does not depend on it.
constexpr int kClusterThreads = 512;
constexpr int kClusterMaxHeadNodes = 4096;
constexpr int kClusterMax = 16;
constexpr int kClusterK0 = 576 + 800;  // K0 and its regrouped copy (floats)

__device__ __forceinline__ unsigned cluster_ctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_nctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
// generic address of p (this CTA's shared memory) in CTA `rank` of the cluster
__device__ __forceinline__ const float *cl_map(const float *p, int rank) {
    uint64_t r;
    asm("mapa.u64 %0, %1, %2;" : "=l"(r) : "l"(reinterpret_cast<uint64_t>(p)), "r"(rank));
    return reinterpret_cast<const float *>(r);
}
// n / d for the level's small divisors by one rounded product (exact for every n
// of the level: the host checks each reciprocal against integer division)
__device__ __forceinline__ int cl_div(int n, float r) {
    return __float2int_rz(__fmul_rn(__fadd_rn(__int2float_rn(n), 0.5f), r));
}
__device__ __forceinline__ void cl_ijk(const ClusterLevel &L, int n, int &i, int &j, int &k) {
    k = cl_div(n, L.rNXY);
    const int rem = n - k * L.NXY;
    j = cl_div(rem, L.rNX);
    i = rem - j * L.NX;
}
// component c of node n of a vector whose slabs sit at `slab` in every CTA: a
// plain load through the generic window, so that independent loads overlap
__device__ __forceinline__ float cl_get(const float *slab, const ClusterLevel &L, int n, int c, int rank) {
    const int owner = cl_div(n, L.rchunk);
    const float *p = slab + (n - owner * L.chunk) * 3 + c;
    return owner == rank ? *p : *cl_map(p, owner);
}

enum { kClX = 0, kClB, kClR, kClD, kClY };
__device__ __forceinline__ float *cl_slab(float *sm, const ClusterLevel &L, int v) {
    return sm + L.s_vec + v * 3 * L.chunk;
}

// One phase of the cluster V-cycle on level L: y = A in with eight lanes per node
// (as bottom_apply), the elementwise update that follows it done by the lanes that
// hold each dof's sum, so that the phase needs no second barrier:
//   STEP 0, residual:             in = x;   r = b - y
//   STEP 1, first smoothing step: in = D^-1 rin theta (formed while staging rin);
//           r0 = rin, d0 = D^-1 r0 theta, x0 = d0 or x + d0, then the step-1 update
//   STEP 2, later smoothing step: in = d;   r -= y, d' = c1 d + c2 D^-1 r, x += d'
// (0 on Dirichlet dofs throughout).  The operand over the CTA's nodes and their
// one-layer halo (nodes n0 - H .. n1 - 1 + H, H = NX NY + NX + 1) is first staged
// in shared memory; no phase writes a slab that another CTA reads in it (the
// callers rotate r, d and y).
struct ClusterStep {
    const float *in, *b, *r_src, *d_src;  // slabs (this CTA's shared memory)
    float *r_dst, *d_dst, *x;
    bool x0_zero;
    float inv_theta, c1, c2;
};

template <int STEP>
__device__ void cl_step(const ClusterLevel &L, float *sm, const float *sK, float *stage, const ClusterStep &S,
                        int rank) {
    const int nn = L.NX * L.NY * L.NZ;
    const int n0 = rank * L.chunk, n1 = min(nn, n0 + L.chunk);
    const int H = L.NX * L.NY + L.NX + 1;
    const float *dinvL = sm + L.s_dinv, *EL = sm + L.s_E;
    const int nlo = max(0, n0 - H);
    if (n0 < n1) {
        const int cnt = 3 * (min(nn - 1, n1 - 1 + H) - nlo + 1);
        for (int t = threadIdx.x; t < cnt; t += kClusterThreads) {
            const int n = nlo + t / 3, c = t - 3 * (t / 3);
            const float v = cl_get(S.in, L, n, c, rank);
            stage[t] = STEP == 1 ? dinvL[3 * n + c] * v * S.inv_theta : v;
        }
    }
    __syncthreads();
    const int corner = threadIdx.x & 7;
    const int dx = corner & 1, dy = (corner >> 1) & 1, dz = corner >> 2;
    const float4 *Kt = reinterpret_cast<const float4 *>(sK + 576 + 100 * corner_index(dx, dy, dz));
    for (int base = n0; base < n1; base += kClusterThreads / 8) {
        const int n = base + (threadIdx.x >> 3);
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
        if (n < n1) {
            int i, j, k;
            cl_ijk(L, n, i, j, k);
            const int ex = i - dx, ey = j - dy, ez = k - dz;
            if (ex >= 0 && ey >= 0 && ez >= 0 && ex < L.nx && ey < L.ny && ez < L.nz) {
                const float e = EL[ex + L.nx * (ey + L.ny * ez)];
                const float *u0p = stage + 3 * (ex + L.NX * (ey + L.NY * ez) - nlo);
                float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
#pragma unroll
                for (int bc = 0; bc < 8; bc++) {
                    int bx, by, bz;
                    corner_bits(bc, bx, by, bz);
                    const float *u = u0p + 3 * (bx + L.NX * (by + L.NY * bz));
                    const float4 k0 = Kt[3 * bc], k1 = Kt[3 * bc + 1], k2 = Kt[3 * bc + 2];
                    s0 = fmaf(k0.z, u[2], fmaf(k0.y, u[1], fmaf(k0.x, u[0], s0)));
                    s1 = fmaf(k1.y, u[2], fmaf(k1.x, u[1], fmaf(k0.w, u[0], s1)));
                    s2 = fmaf(k2.x, u[2], fmaf(k1.w, u[1], fmaf(k1.z, u[0], s2)));
                }
                a0 = e * s0;
                a1 = e * s1;
                a2 = e * s2;
            }
        }
#pragma unroll
        for (int off = 1; off < 8; off <<= 1) {
            a0 += __shfl_xor_sync(0xffffffffu, a0, off);
            a1 += __shfl_xor_sync(0xffffffffu, a1, off);
            a2 += __shfl_xor_sync(0xffffffffu, a2, off);
        }
        if (n < n1 && corner < 3) {
            const int lo = 3 * (n - n0) + corner;
            const float dn = dinvL[3 * n + corner];
            const float y = dn == 0.0f ? 0.0f : (corner == 0 ? a0 : (corner == 1 ? a1 : a2));
            if (STEP == 0) {
                S.r_dst[lo] = dn == 0.0f ? 0.0f : S.b[lo] - y;
            } else {
                const float rv0 = S.r_src[lo];
                float d0, x0;
                if (STEP == 1) {
                    d0 = dn * rv0 * S.inv_theta;
                    x0 = S.x0_zero ? d0 : S.x[lo] + d0;
                } else {
                    d0 = S.d_src[lo];
                    x0 = S.x[lo];
                }
                const float rv = rv0 - y;
                const float dv = fmaf(S.c1, d0, S.c2 * dn * rv);
                S.r_dst[lo] = rv;
                S.d_dst[lo] = dv;
                S.x[lo] = x0 + dv;
            }
        }
    }
}

// x (+)= Chebyshev-Jacobi smoothing of degree deg for rhs rin (as bottom_smooth):
// deg - 1 phases (one for deg = 1); r, d and y are rotated so that no phase
// writes what other CTAs read in it
__device__ void cl_smooth(const ClusterLevel &L, float *sm, const float *sK, float *stage, const float *rin,
                          bool x0_zero, int deg, float inv_theta, const float *c1, const float *c2, int rank) {
    float *x = cl_slab(sm, L, kClX), *r = cl_slab(sm, L, kClR), *d = cl_slab(sm, L, kClD),
          *sp = cl_slab(sm, L, kClY);
    if (deg <= 1) {
        const int nn = L.NX * L.NY * L.NZ;
        const int n0 = rank * L.chunk, nown = max(0, min(nn, n0 + L.chunk) - n0);
        const float *dinvL = sm + L.s_dinv + 3 * n0;
        for (int q = threadIdx.x; q < 3 * nown; q += kClusterThreads) {
            const float rv = rin[q], dv = dinvL[q] * rv * inv_theta;
            r[q] = rv;
            d[q] = dv;
            x[q] = x0_zero ? dv : x[q] + dv;
        }
        cluster_barrier();
        return;
    }
    ClusterStep S{};
    S.x = x;
    S.inv_theta = inv_theta;
    S.x0_zero = x0_zero;
    // step 1 reads rin at the neighbours: its residual goes to the spare slab when rin is r
    S.in = rin;
    S.r_src = rin;
    S.r_dst = rin == r ? sp : r;
    S.d_dst = d;
    S.c1 = c1[1];
    S.c2 = c2[1];
    cl_step<1>(L, sm, sK, stage, S, rank);
    cluster_barrier();
    if (rin == r) {
        float *t = r; r = sp; sp = t;
    }
    for (int k = 2; k < deg; k++) {
        // reads d at the neighbours: the new direction goes to the spare slab
        S.in = d;
        S.r_src = r;
        S.r_dst = r;
        S.d_src = d;
        S.d_dst = sp;
        S.c1 = c1[k];
        S.c2 = c2[k];
        cl_step<2>(L, sm, sK, stage, S, rank);
        cluster_barrier();
        float *t = d; d = sp; sp = t;
    }
}

// r = b - A x (0 on Dirichlet dofs), one phase
__device__ void cl_residual(const ClusterLevel &L, float *sm, const float *sK, float *stage, int rank) {
    ClusterStep S{};
    S.in = cl_slab(sm, L, kClX);
    S.b = cl_slab(sm, L, kClB);
    S.r_dst = cl_slab(sm, L, kClR);
    cl_step<0>(L, sm, sK, stage, S, rank);
    cluster_barrier();
}

__global__ void __launch_bounds__(kClusterThreads, 1) mg_bottom_cluster_kernel(
    const ClusterChain *__restrict__ chains, const MfState *states, const float *__restrict__ E32,
    const float *__restrict__ dinv, const float *__restrict__ mb, float *__restrict__ mx,
    const float *__restrict__ k0f, BottomCheb cc, int sdeg, int cdeg, const int64_t *__restrict__ coarse_off,
    const float *__restrict__ coarse_inv, const int *__restrict__ coarse_ok) {
    // D^-1, the moduli and the coarse inverse were formed before this graph ran
    // (activation); they are loaded while the preceding kernel finishes, the
    // head's rhs and the solver state only after it
    pdl_trigger();
    extern __shared__ __align__(16) float sm[];  // K0 tables, stage, per level: D^-1, E, slabs
    __shared__ ClusterChain sc;
    const int csize = (int)cluster_nctarank(), rank = (int)cluster_ctarank();
    const int chain = blockIdx.x / csize;
    {
        const int *src = reinterpret_cast<const int *>(chains + chain);
        int *dst = reinterpret_cast<int *>(&sc);
        for (int i = threadIdx.x; i < (int)(sizeof(ClusterChain) / 4); i += kClusterThreads) dst[i] = src[i];
    }
    for (int i = threadIdx.x; i < kClusterK0; i += kClusterThreads) sm[i] = k0f[i];
    __syncthreads();
    const int m = sc.m;
    const float *sK = sm;
    float *stage = sm + sc.s_stage;
    // D^-1 and E of every level (compact order), the head's rhs over this CTA's nodes
    for (int l = 0; l < m; l++) {
        const ClusterLevel &L = sc.L[l];
        const int nn = L.NX * L.NY * L.NZ, ne = L.nx * L.ny * L.nz;
        for (int q = threadIdx.x; q < 3 * nn; q += kClusterThreads) {
            const int n = q / 3, c = q - 3 * n;
            const int i = n % L.NX, j = (n / L.NX) % L.NY, k = n / (L.NX * L.NY);
            sm[L.s_dinv + q] = dinv[L.dof_off + ((int64_t)k * L.NY + j) * L.pitch + 3 * i + c];
        }
        for (int e = threadIdx.x; e < ne; e += kClusterThreads) {
            const int ex = e % L.nx, ey = (e / L.nx) % L.ny, ez = e / (L.nx * L.ny);
            sm[L.s_E + e] = E32[L.elem_off + ((int64_t)ez * L.ny + ey) * L.pitch_e + ex];
        }
    }
    // the direct solve's rows of this CTA (one warp per row), loaded now
    const ClusterLevel &Lc = sc.L[m - 1];
    const int64_t inv_off = coarse_ok[chain] ? coarse_off[chain] : -1;
    const int nnc = Lc.NX * Lc.NY * Lc.NZ, ndc = 3 * nnc;
    const int c0 = rank * Lc.chunk, crows = 3 * max(0, min(nnc, c0 + Lc.chunk) - c0);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kInvPer = (kCoarseDirectMax + 31) / 32;
    float inv[kInvPer];
#pragma unroll
    for (int t = 0; t < kInvPer; t++) {
        const int r = lane + 32 * t;
        inv[t] = (inv_off >= 0 && warp < crows && r < ndc)
                     ? __ldg(coarse_inv + inv_off + (int64_t)(3 * c0 + warp) * ndc + r)
                     : 0.0f;
    }
    const ClusterLevel &L0 = sc.L[0];
    pdl_wait();
    // the same state in every CTA of the cluster: all return, or none
    if (states[sc.root].done) return;
    {
        const int nn = L0.NX * L0.NY * L0.NZ, n0 = rank * L0.chunk, nown = max(0, min(nn, n0 + L0.chunk) - n0);
        float *b0 = cl_slab(sm, L0, kClB);
        for (int q = threadIdx.x; q < 3 * nown; q += kClusterThreads) {
            const int n = n0 + q / 3, c = q - 3 * (q / 3);
            int i, j, k;
            cl_ijk(L0, n, i, j, k);
            b0[q] = __ldcg(mb + L0.dof_off + ((int64_t)k * L0.NY + j) * L0.pitch + 3 * i + c);
        }
    }
    cluster_barrier();  // every CTA's tables and rhs are in place
    // down: smooth, residual, restrict
    for (int l = 0; l < m - 1; l++) {
        const ClusterLevel &F = sc.L[l], &C = sc.L[l + 1];
        cl_smooth(F, sm, sK, stage, cl_slab(sm, F, kClB), true, sdeg, cc.inv_theta_s, cc.c1s, cc.c2s, rank);
        cl_residual(F, sm, sK, stage, rank);
        // one warp per coarse node: lane t < 27 takes fine neighbour t (all three
        // components), the weighted values meet in a fixed xor butterfly
        const int nnC = C.NX * C.NY * C.NZ, n0 = rank * C.chunk, n1 = min(nnC, n0 + C.chunk);
        const float *rF = cl_slab(sm, F, kClR);
        float *bC = cl_slab(sm, C, kClB);
        const int warp_r = threadIdx.x >> 5, lane_r = threadIdx.x & 31;
        for (int n = n0 + warp_r; n < n1; n += kClusterThreads / 32) {
            int I, J, K;
            cl_ijk(C, n, I, J, K);
            const int dx = lane_r % 3 - 1, dy = (lane_r / 3) % 3 - 1, dz = lane_r / 9 - 1;
            const int ii = 2 * I + dx, jj = 2 * J + dy, kk = 2 * K + dz;
            float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f;
            if (lane_r < 27 && ii >= 0 && ii < F.NX && jj >= 0 && jj < F.NY && kk >= 0 && kk < F.NZ) {
                const int nf = ii + F.NX * (jj + F.NY * kk);
                const float w = (dz ? 0.5f : 1.0f) * (dy ? 0.5f : 1.0f) * (dx ? 0.5f : 1.0f);
                v0 = w * cl_get(rF, F, nf, 0, rank);
                v1 = w * cl_get(rF, F, nf, 1, rank);
                v2 = w * cl_get(rF, F, nf, 2, rank);
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                v0 += __shfl_xor_sync(0xffffffffu, v0, off);
                v1 += __shfl_xor_sync(0xffffffffu, v1, off);
                v2 += __shfl_xor_sync(0xffffffffu, v2, off);
            }
            if (lane_r < 3) {
                const float v = lane_r == 0 ? v0 : (lane_r == 1 ? v1 : v2);
                bC[3 * (n - n0) + lane_r] = sm[C.s_dinv + 3 * n + lane_r] != 0.0f ? v : 0.0f;
            }
        }
        cluster_barrier();
    }
    // coarsest grid of the chain: exact solve with the stored inverse, or smoothing
    if (inv_off >= 0) {
        // one warp per own row, partial sums met by a fixed xor butterfly; the
        // first pass uses the rows loaded at the start
        const float *bc = cl_slab(sm, Lc, kClB);
        float *xc = cl_slab(sm, Lc, kClX);
        for (int w0 = 0; w0 < crows; w0 += kClusterThreads / 32) {
            const int w = w0 + warp;
            if (w >= crows) break;  // whole warps leave together
            float sacc = 0.0f;
#pragma unroll
            for (int t = 0; t < kInvPer; t++) {
                const int r = lane + 32 * t;
                if (r < ndc) {
                    const float a = w0 == 0 ? inv[t] : __ldg(coarse_inv + inv_off + (int64_t)(3 * c0 + w) * ndc + r);
                    sacc = fmaf(a, cl_get(bc, Lc, r / 3, r - 3 * (r / 3), rank), sacc);
                }
            }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, off);
            if (lane == 0) xc[w] = sm[Lc.s_dinv + 3 * c0 + w] == 0.0f ? 0.0f : sacc;
        }
        cluster_barrier();
    } else {
        cl_smooth(Lc, sm, sK, stage, cl_slab(sm, Lc, kClB), true, cdeg, cc.inv_theta_c, cc.c1c, cc.c2c, rank);
    }
    // up: prolong, residual, post-smooth
    for (int l = m - 2; l >= 0; l--) {
        const ClusterLevel &F = sc.L[l], &C = sc.L[l + 1];
        const int nnF = F.NX * F.NY * F.NZ, n0 = rank * F.chunk, nown = max(0, min(nnF, n0 + F.chunk) - n0);
        const float *xC = cl_slab(sm, C, kClX);
        float *xF = cl_slab(sm, F, kClX);
        for (int q = threadIdx.x; q < 3 * nown; q += kClusterThreads) {
            const int n = n0 + q / 3, c = q - 3 * (q / 3);
            if (sm[F.s_dinv + 3 * n + c] == 0.0f) continue;
            int ii, jj, kk;
            cl_ijk(F, n, ii, jj, kk);
            const float w = ((ii & 1) ? 0.5f : 1.0f) * ((jj & 1) ? 0.5f : 1.0f) * ((kk & 1) ? 0.5f : 1.0f);
            // the 1, 2, 4 or 8 parents' loads first, then the sums in a fixed order
            float v[8];
#pragma unroll
            for (int t = 0; t < 8; t++) {
                const int a = t >> 2, bb = (t >> 1) & 1, cc2 = t & 1;
                const bool use = (a == 0 || (kk & 1)) && (bb == 0 || (jj & 1)) && (cc2 == 0 || (ii & 1));
                v[t] = use ? cl_get(xC, C, ((ii + cc2) >> 1) + C.NX * (((jj + bb) >> 1) + C.NY * ((kk + a) >> 1)), c, rank)
                           : 0.0f;
            }
            float acc = 0.0f;
#pragma unroll
            for (int t = 0; t < 8; t++) {
                const int a = t >> 2, bb = (t >> 1) & 1, cc2 = t & 1;
                if ((a == 0 || (kk & 1)) && (bb == 0 || (jj & 1)) && (cc2 == 0 || (ii & 1))) acc = fmaf(w, v[t], acc);
            }
            xF[q] += acc;
        }
        cluster_barrier();
        cl_residual(F, sm, sK, stage, rank);
        // post-smoothing on the residual: x += S(r) (the smoother starts from r in place)
        cl_smooth(F, sm, sK, stage, cl_slab(sm, F, kClR), false, sdeg, cc.inv_theta_s, cc.c1s, cc.c2s, rank);
    }
    // the head's correction over this CTA's nodes back to the padded global layout
    {
        const int nn = L0.NX * L0.NY * L0.NZ, n0 = rank * L0.chunk, nown = max(0, min(nn, n0 + L0.chunk) - n0);
        const float *x0 = cl_slab(sm, L0, kClX);
        for (int q = threadIdx.x; q < 3 * nown; q += kClusterThreads) {
            const int n = n0 + q / 3, c = q - 3 * (q / 3);
            int i, j, k;
            cl_ijk(L0, n, i, j, k);
            mx[L0.dof_off + ((int64_t)k * L0.NY + j) * L0.pitch + 3 * i + c] = x0[q];
        }
    }
}

// inner CG start (problems in INIT): b = scale r64 (unit norm), x = 0, r = b,
// z = D^-1 r, p0 = p1 = 0; moves the problem to CG
__global__ void __launch_bounds__(kThreads) mf_inner_init_kernel(
    const MfChunkDesc *__restrict__ chunks, int n_chunks, const MfProblem *__restrict__ probs,
    const double *__restrict__ r64, float *__restrict__ x, float *__restrict__ r,
    float *__restrict__ z, float *__restrict__ p0, float *__restrict__ p1,
    const float *__restrict__ dinv, MfState *states, double *__restrict__ chunk_part,
    double inner_rtol2, int maxit) {
    pdl_enter();
    __shared__ double red_sh[kThreads / 32];
    __shared__ int sh_last;
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x) {
        const MfChunkDesc C = chunks[ci];
        MfState *st = states + C.prob;
        if (st->phase != kPhaseInit) continue;
        const double scale = st->scale;
        float rz = 0.0f, rr = 0.0f;
        for (int64_t i = C.begin + threadIdx.x; i < C.end; i += kThreads) {
            const float bi = dinv[i] != 0.0f ? (float)(r64[i] * scale) : 0.0f;
            x[i] = 0.0f;
            r[i] = bi;
            const float zi = dinv[i] * bi;
            z[i] = zi;
            p0[i] = 0.0f;  // either may be the first step's p_old
            p1[i] = 0.0f;
            rz = fmaf(bi, zi, rz);
            rr = fmaf(bi, bi, rr);
        }
        const double srz = block_sum_f(rz, red_sh);
        const double srr = block_sum_f(rr, red_sh);
        const MfProblem &P = probs[C.prob];
        if (threadIdx.x == 0) {
            chunk_part[ci] = srz;
            chunk_part[n_chunks + ci] = srr;
            __threadfence();
            const unsigned t = atomicAdd(&st->cnt_update, 1u);
            sh_last = (t == (unsigned)P.chunk_count - 1);
        }
        __syncthreads();
        if (sh_last) {
            const double trz = ordered_sum(chunk_part, P.chunk_begin, P.chunk_count);
            const double trr = ordered_sum(chunk_part + n_chunks, P.chunk_begin, P.chunk_count);
            if (threadIdx.x == 0) {
                st->cnt_update = 0;
                st->rz = trz;
                st->rr = trr;
                st->bb = trr;
                st->tol2 = inner_rtol2 * trr;
                st->beta = 0.0;
                st->iter = 0;
                st->maxit = maxit;
                st->status = 0;
                st->first = 1;
                st->done = (trr <= st->tol2 || trr == 0.0) ? 1 : 0;
                if (is_bad(trr)) { st->status = MG_ENAN; st->done = 1; }
                st->phase = kPhaseCG;
            }
        }
        __syncthreads();
    }
}

// a problem whose inner CG has just stopped and whose correction is usable
__device__ __forceinline__ bool inner_finished(const MfState *st) {
    return st->phase == kPhaseCG && st->done && (st->status == 0 || st->status == MG_ENOCONV);
}

// refinement update u += x / scale (x is 0 on Dirichlet dofs and padding) for
// the problems whose inner CG has stopped
__global__ void mf_refine_kernel(const MfChunkDesc *__restrict__ chunks, int n_chunks,
                                 const float *__restrict__ x, double *__restrict__ u64,
                                 const MfState *states) {
    pdl_enter();
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x) {
        const MfChunkDesc C = chunks[ci];
        const MfState *st = states + C.prob;
        if (!inner_finished(st)) continue;
        const double inv = 1.0 / st->scale;
        for (int64_t i = C.begin + threadIdx.x; i < C.end; i += blockDim.x)
            u64[i] = fma((double)x[i], inv, u64[i]);
    }
}

// after the refinement update: a stopped inner CG sends its problem back to the
// FP64 residual, or ends it on a breakdown / NaN (one thread per problem)
__global__ void mf_phase_kernel(MfState *states, int n_fine) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_fine) return;
    MfState *st = states + i;
    if (st->phase != kPhaseCG || !st->done) return;
    if (st->status != 0 && st->status != MG_ENOCONV) {
        st->ref_status = st->status;
        st->ref_done = 1;
        st->phase = kPhaseFin;
    } else {
        st->refine += 1;
        st->status = 0;
        st->u_zero = 0;  // u has been corrected
        st->phase = kPhaseResid;
    }
}

// FP64 outer residual r = f - K u (CUDA-core FP64, factored element stiffness,
// hex8_factored.cuh), per-problem ||r||^2 -> scale.  A brick of kBN^3 owned
// nodes evaluates its (kBN+1)^3 surrounding elements in three groups of kBE/3
// element layers: each element's 24 corner results go to shared memory, then
// every owned node adds the results of its elements in that group to register
// accumulators, in a fixed order (deterministic, atomic-free).
constexpr int kRGroupLayers = kBE / 3;                      // 3 element layers per group
constexpr int kRGroupEl = kBE * kBE * kRGroupLayers;        // 243 elements
constexpr int kRNodesPerThread = (kBN * kBN * kBN + kThreads - 1) / kThreads;  // 2
constexpr int kOffU64 = 0;
constexpr int kOffE64 = kBU * kBU * kBU * 3 * 8;            // 24000
constexpr int kOffY64 = kOffE64 + kNEL * 8;                 // +5832
constexpr int kResidSmem = kOffY64 + 24 * kRGroupEl * 8;    // +46656
static_assert(kBE % 3 == 0 && kRGroupEl <= kThreads, "one element per thread and group");

__global__ void __launch_bounds__(kThreads) mf_residual64_kernel(
    const MfProblem *__restrict__ probs, const MfBrick *__restrict__ bricks, int n_bricks,
    const dfloat *__restrict__ Edf, const uint8_t *__restrict__ node_fix,
    const double *__restrict__ u64, const double *__restrict__ f64, const FacK<dfloat> K,
    double *__restrict__ r64, MfState *states, double *__restrict__ brick_part, double rtol2,
    int max_ref) {
    pdl_enter();
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ double red_sh[kThreads / 32];
    __shared__ int sh_last;
    dfloat *su = reinterpret_cast<dfloat *>(smem + kOffU64);
    dfloat *sE = reinterpret_cast<dfloat *>(smem + kOffE64);
    dfloat(*sY)[kRGroupEl] = reinterpret_cast<dfloat(*)[kRGroupEl]>(smem + kOffY64);  // [b * 3 + c][element]
    for (int bi = blockIdx.x; bi < n_bricks; bi += gridDim.x) {
        const MfBrick br = bricks[bi];
        const MfProblem P = probs[br.prob];
        MfState *st = states + br.prob;
        if (st->phase != kPhaseResid) continue;
        const bool need_ff = st->ff64 == 0.0;  // first residual of a solve: also ||f||^2
        const bool u_zero = st->u_zero != 0;    // cold start: r = f, no operator pass
        const int gx0 = br.bx * kBN, gy0 = br.by * kBN, gz0 = br.bz * kBN;
        __syncthreads();
        for (int i = threadIdx.x; i < (u_zero ? 0 : kBU * kBU * kBU * 3); i += kThreads) {
            const int node = i / 3, c = i - node * 3;
            const int ux = node % kBU, uy = (node / kBU) % kBU, uz = node / (kBU * kBU);
            const int gx = gx0 - 1 + ux, gy = gy0 - 1 + uy, gz = gz0 - 1 + uz;
            double v = 0.0;
            if (gx >= 0 && gx < P.NX && gy >= 0 && gy < P.NY && gz >= 0 && gz < P.NZ) {
                const int64_t gn = gx + (int64_t)P.NX * (gy + (int64_t)P.NY * gz);
                if (!((node_fix[P.node_off + gn] >> c) & 1)) v = u64[dof_index(P, gx, gy, gz, c)];
            }
            su[i] = df_split(v);
        }
        for (int l = threadIdx.x; l < (u_zero ? 0 : kNEL); l += kThreads) {
            const int ex = l % kBE, ey = (l / kBE) % kBE, ez = l / (kBE * kBE);
            const int gx = gx0 - 1 + ex, gy = gy0 - 1 + ey, gz = gz0 - 1 + ez;
            dfloat e = df_zero();
            if (gx >= 0 && gx < P.nx && gy >= 0 && gy < P.ny && gz >= 0 && gz < P.nz)
                e = Edf[P.elem_off + ((int64_t)gz * P.ny + gy) * P.pitch_e + gx];
            sE[l] = e;
        }
        dfloat acc[kRNodesPerThread][3];
#pragma unroll
        for (int k = 0; k < kRNodesPerThread; k++) acc[k][0] = acc[k][1] = acc[k][2] = df_zero();
        for (int g = 0; g < (u_zero ? 0 : 3); g++) {
            __syncthreads();  // su / sE loaded; the previous group's readers of sY are done
            const int l = threadIdx.x;
            if (l < kRGroupEl) {
                const int ex = l % kBE, ey = (l / kBE) % kBE, ez = g * kRGroupLayers + l / (kBE * kBE);
                const dfloat e = sE[ex + kBE * (ey + kBE * ez)];
                dfloat v[3][8];
#pragma unroll
                for (int b = 0; b < 8; b++) {
                    const dfloat *ub = su + (((ez + (b >> 2)) * kBU + ey + ((b >> 1) & 1)) * kBU + ex + (b & 1)) * 3;
                    v[0][b] = ub[0]; v[1][b] = ub[1]; v[2][b] = ub[2];
                }
                if (e.hi != 0.0f) {
                    hex8_factored_apply(K, e, v);
                } else {
#pragma unroll
                    for (int b = 0; b < 8; b++) v[0][b] = v[1][b] = v[2][b] = df_zero();
                }
#pragma unroll
                for (int b = 0; b < 8; b++) {
                    sY[b * 3][l] = v[0][b];
                    sY[b * 3 + 1][l] = v[1][b];
                    sY[b * 3 + 2][l] = v[2][b];
                }
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < kRNodesPerThread; k++) {
                const int node = threadIdx.x + k * kThreads;
                if (node >= kBN * kBN * kBN) continue;
                const int ox = node % kBN, oy = (node / kBN) % kBN, oz = node / (kBN * kBN);
#pragma unroll
                for (int b = 0; b < 8; b++) {  // the node is corner b of element (o + 1 - d)
                    const int dx = b & 1, dy = (b >> 1) & 1, dz = b >> 2;
                    const int lz = oz + 1 - dz - g * kRGroupLayers;
                    if (lz < 0 || lz >= kRGroupLayers) continue;
                    const int el = (ox + 1 - dx) + kBE * ((oy + 1 - dy) + kBE * lz);
                    acc[k][0] += sY[b * 3][el];
                    acc[k][1] += sY[b * 3 + 1][el];
                    acc[k][2] += sY[b * 3 + 2][el];
                }
            }
        }
        double part = 0.0, fpart = 0.0;
#pragma unroll
        for (int k = 0; k < kRNodesPerThread; k++) {
            const int node = threadIdx.x + k * kThreads;
            if (node >= kBN * kBN * kBN) continue;
            const int ox = node % kBN, oy = (node / kBN) % kBN, oz = node / (kBN * kBN);
            const int gx = gx0 + ox, gy = gy0 + oy, gz = gz0 + oz;
            if (gx >= P.NX || gy >= P.NY || gz >= P.NZ) continue;
            const int64_t gn = gx + (int64_t)P.NX * (gy + (int64_t)P.NY * gz);
            const uint8_t fix = node_fix[P.node_off + gn];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int64_t gd = dof_index(P, gx, gy, gz, c);
                const double fv = f64[gd];
                double rv = fv - df_to(acc[k][c]);
                if ((fix >> c) & 1) rv = 0.0;
                r64[gd] = rv;
                part = fma(rv, rv, part);
                fpart = fma(fv, fv, fpart);
            }
        }
        const double s = block_sum(part, red_sh);
        const double sf = need_ff ? block_sum(fpart, red_sh) : 0.0;
        if (threadIdx.x == 0) {
            brick_part[bi] = s;
            brick_part[n_bricks + bi] = sf;
            __threadfence();
            const unsigned t = atomicAdd(&st->cnt_res, 1u);
            sh_last = (t == (unsigned)P.brick_count - 1);
        }
        __syncthreads();
        if (sh_last) {
            const double rr = ordered_sum(brick_part, P.brick_begin, P.brick_count);
            const double ff = need_ff ? ordered_sum(brick_part + n_bricks, P.brick_begin, P.brick_count) : 0.0;
            if (threadIdx.x == 0) {
                st->cnt_res = 0;
                if (need_ff) st->ff64 = ff > 0.0 ? ff : -1.0;  // -1: zero load (u = 0)
                st->rr64 = rr;
                st->scale = rr > 0.0 ? 1.0 / sqrt(rr) : 1.0;
                st->phase = kPhaseFin;
                st->ref_done = 1;
                if (st->ff64 < 0.0) st->rr64 = 0.0;
                else if (is_bad(rr)) st->ref_status = MG_ENAN;
                else if (rr <= rtol2 * st->ff64) st->ref_status = 0;
                else if (st->refine >= max_ref) st->ref_status = MG_ENOCONV;
                else { st->ref_done = 0; st->phase = kPhaseInit; }
            }
        }
        __syncthreads();
    }
}

// Jacobi inverse of the mixed operator: 1 / sum_e E_e K0[3a+c][3a+c];
// 0 on Dirichlet dofs and padding (marks them for the vector kernels)
__global__ void mf_diag_kernel(const MfProblem *__restrict__ probs, const int *__restrict__ list,
                               const float *__restrict__ E32, const uint8_t *__restrict__ node_fix,
                               const double *__restrict__ K0, float *__restrict__ dinv) {
    const int pi = list ? list[blockIdx.y] : (int)blockIdx.y;
    const MfProblem P = probs[pi];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n_pad;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = i / P.pitch;
        const int xin = (int)(i - row * P.pitch);
        float out = 0.0f;
        if (xin < 3 * P.NX) {
            const int gx = xin / 3, c = xin - 3 * gx;
            const int gy = (int)(row % P.NY), gz = (int)(row / P.NY);
            const int64_t gn = gx + (int64_t)P.NX * (gy + (int64_t)P.NY * gz);
            // FP32 (the Jacobi inverse is stored in FP32; GB300's FP64 pipe issues two
            // DFMA per cycle per SM), the node's elements in a fixed order
            float d = 0.0f;
            for (int dz = 0; dz < 2; dz++)
                for (int dy = 0; dy < 2; dy++)
                    for (int dx = 0; dx < 2; dx++) {
                        const int ex = gx - dx, ey = gy - dy, ez = gz - dz;
                        if (ex < 0 || ey < 0 || ez < 0 || ex >= P.nx || ey >= P.ny || ez >= P.nz) continue;
                        const int k = 3 * corner_index(dx, dy, dz) + c;
                        d = fmaf(E32[P.elem_off + ((int64_t)ez * P.ny + ey) * P.pitch_e + ex], (float)K0[k * 24 + k], d);
                    }
            const bool fixed = (node_fix[P.node_off + gn] >> c) & 1;
            out = (fixed || d == 0.0f) ? 0.0f : 1.0f / d;
        }
        dinv[P.dof_off + i] = out;
    }
}

// compliance adjoint sensitivity dC/drho_e = -dE_e u_e^T K0 u_e, written
// unpadded (element order x-fastest) at dc + out_off[prob]
// dc_e = -dE_e u_e^T K0 u_e for the listed problems, in the factored form:
// u_e^T K0 u_e = u~^T (Khat / 64) u~ with u~ the sum/difference modes of u_e (72
// butterfly additions, 45 + 21 products instead of the 600 of the dense product),
// in double-float arithmetic on the FP32 pipes (48-bit significand; GB300's FP64
// pipe issues two DFMA per cycle per SM) from the FP64 u and Khat, the final
// product with dE_e in FP64
__global__ void mf_sens_kernel(const MfProblem *__restrict__ probs, int n_probs,
                               const double *__restrict__ dE64, const uint8_t *__restrict__ node_fix,
                               const double *__restrict__ u64, FacK<dfloat> K,
                               const int64_t *__restrict__ out_off, double *__restrict__ dc) {
    const int pi = blockIdx.y;
    if (pi >= n_probs) return;
    const MfProblem P = probs[pi];
    if (out_off[pi] < 0) return;  // not part of this evaluation
    const int64_t ne = (int64_t)P.nx * P.ny * P.nz;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int ex = (int)(e % P.nx), ey = (int)((e / P.nx) % P.ny), ez = (int)(e / ((int64_t)P.nx * P.ny));
        dfloat v[3][8];  // component c at lexicographic corner b = bx + 2 by + 4 bz
#pragma unroll
        for (int b = 0; b < 8; b++) {
            const int bx = b & 1, by = (b >> 1) & 1, bz = b >> 2;
            const int64_t gn = (ex + bx) + (int64_t)P.NX * ((ey + by) + (int64_t)P.NY * (ez + bz));
            const uint8_t fx = node_fix[P.node_off + gn];
            const double *u = u64 + dof_index(P, ex + bx, ey + by, ez + bz, 0);
#pragma unroll
            for (int c = 0; c < 3; c++) v[c][b] = ((fx >> c) & 1) ? df_zero() : df_split(u[c]);
        }
        hex8_factored_forward(v);
        dfloat yh[3][8];
        hex8_factored_khat(K, v, yh);
        dfloat s = df_zero();
#pragma unroll
        for (int c = 0; c < 3; c++)
#pragma unroll
            for (int m = 1; m < 8; m++) s = fma_t(v[c][m], yh[c][m], s);
        dc[out_off[pi] + e] = -dE64[P.elem_off + ((int64_t)ez * P.ny + ey) * P.pitch_e + ex] * df_to(s);
    }
}

// per-chunk partial of a.b; host sums each problem's chunks in order
__global__ void mf_dot_chunks_kernel(const MfChunkDesc *__restrict__ chunks, int n_chunks,
                                     const double *__restrict__ a, const double *__restrict__ b,
                                     double *__restrict__ part) {
    __shared__ double red_sh[kThreads / 32];
    for (int ci = blockIdx.x; ci < n_chunks; ci += gridDim.x) {
        const MfChunkDesc C = chunks[ci];
        double s = 0.0;
        for (int64_t i = C.begin + threadIdx.x; i < C.end; i += kThreads) s = fma(a[i], b[i], s);
        const double t = block_sum(s, red_sh);
        if (threadIdx.x == 0) part[ci] = t;
        __syncthreads();
    }
}

// unpadded element array (x-fastest) -> padded FP32, double-float (the outer
// residual's moduli) and FP64 (dE/drho) tables of problem P
__global__ void pack_elems_kernel(const MfProblem *__restrict__ probs, int pi,
                                  const double *__restrict__ E, const double *__restrict__ dE,
                                  float *__restrict__ E32, dfloat *__restrict__ Edf,
                                  double *__restrict__ dE64) {
    const MfProblem P = probs[pi];
    const int64_t ne = (int64_t)P.nx * P.ny * P.nz;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ex = e % P.nx, row = e / P.nx;
        const int64_t o = P.elem_off + row * P.pitch_e + ex;
        if (E) {
            Edf[o] = df_from(E[e]);
            E32[o] = (float)E[e];
        }
        if (dE) dE64[o] = dE[e];
    }
}

// padded <-> unpadded node-interleaved FP64 vectors of problem P
__global__ void unpack_vec_kernel(const MfProblem *__restrict__ probs, int pi,
                                  double *__restrict__ padded, double *__restrict__ flat,
                                  int to_flat) {
    const MfProblem P = probs[pi];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n_dofs;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = i / (3 * P.NX), xin = i - row * 3 * P.NX;
        const int64_t o = P.dof_off + row * P.pitch + xin;
        if (to_flat) flat[i] = padded[o];
        else padded[o] = flat[i];
    }
}

__global__ void fill_f32_kernel(float *__restrict__ a, const float *__restrict__ mask, float v,
                                int64_t n) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (mask[i] != 0.0f) ? v : 0.0f;
}

inline unsigned blocks_for(int64_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// K0 in the UMMA K-major no-swizzle layout (B operand, N = 32 rows, zero padded):
// [tf32 hi 768 | tf32 lo 768 | bf16 hi 512 | bf16 lo 512] 32-bit words
// B tiles of the column operator: tile t = dy + 2 dz holds the K0 columns of the
// corners (0, dy, dz) and (1, dy, dz) (K chunk dx: x, y, z, 0 in TF32; x, y, z
// and five zeros in BF16) for the 32 N rows n = 3 a + c (libMesh corner a; rows
// 24..31 zero), in the no-swizzle K-major layout: core matrix (n / 8, dx) at
// ((n / 8) * 2 + dx) * 128 bytes.  [tf32 hi | tf32 lo | bf16 hi | bf16 lo], 1024
// words each.
void pack_b_columns(const double *K0, std::vector<uint32_t> &out) {
    auto tf32_round = [](float x) -> float {
        uint32_t u;
        memcpy(&u, &x, 4);
        if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;  // nearest, ties away
        float r;
        memcpy(&r, &u, 4);
        return r;
    };
    auto bf16_bits = [](float x) -> uint32_t {
        uint32_t u;
        memcpy(&u, &x, 4);
        return ((u + 0x7fffu + ((u >> 16) & 1u)) >> 16) & 0xffffu;  // nearest even
    };
    auto bits_of = [](uint32_t h) -> float {
        const uint32_t u = h << 16;
        float r;
        memcpy(&r, &u, 4);
        return r;
    };
    auto fbits = [](float x) -> uint32_t {
        uint32_t u;
        memcpy(&u, &x, 4);
        return u;
    };
    out.assign(4096, 0u);
    for (int t = 0; t < 4; t++) {
        const int dy = t & 1, dz = t >> 1;
        for (int n = 0; n < 32; n++)
            for (int dx = 0; dx < 2; dx++) {
                const int a = corner_index(dx, dy, dz);
                const int core = (n / 8) * 2 + dx;
                for (int c = 0; c < 3; c++) {
                    const double v = (n < 24) ? K0[n * 24 + 3 * a + c] : 0.0;
                    // TF32: 4 words per row
                    const int w = t * 256 + core * 32 + (n % 8) * 4 + c;
                    const float h = tf32_round((float)v);
                    out[w] = fbits(h);
                    out[1024 + w] = fbits(tf32_round((float)(v - (double)h)));
                    // BF16: 8 halves per row (x, y, z, 0, 0, 0, 0, 0)
                    const int wb = 2048 + t * 256 + core * 32 + (n % 8) * 4 + c / 2;
                    const uint32_t hb = bf16_bits((float)v);
                    const uint32_t lb = bf16_bits((float)(v - (double)bits_of(hb)));
                    out[wb] |= hb << (16 * (c & 1));
                    out[1024 + wb] |= lb << (16 * (c & 1));
                }
            }
    }
}

// Launch with programmatic dependent launch (the kernel starts with pdl_enter):
// the launch latency of the solver step's kernels overlaps their predecessors.
template <typename... KArgs, typename... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// launch_pdl with a thread-block cluster of csize CTAs along x
template <typename... KArgs, typename... Args>
void launch_cluster_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, int csize, cudaStream_t s,
                        Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    attr[1].id = cudaLaunchAttributeClusterDimension;
    attr[1].val.clusterDim.x = (unsigned)csize;
    attr[1].val.clusterDim.y = 1;
    attr[1].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

struct ApplyArgs {
    int col_lo, col_hi, in_slot, parity;  // column range
    const float *rhs;
    float *y;
    int sel = -1;  // -1 every problem; 0 problems with a coarser level; 1 those without
};

template <int PREC, int MODE>
void launch_apply(MfBatch &b, const ApplyArgs &a) {
    const int nc = a.col_hi - a.col_lo;
    if (nc <= 0) return;
    const int grid = std::max(1, std::min(nc, b.col_grid));
    launch_pdl(mf_col_kernel<PREC, MODE>, grid, kColThreads, kColSmem, b.stream, 
        b.probs, b.cols, a.col_lo, a.col_hi, a.sel, b.tmaps, a.in_slot, a.parity, b.Bop2, b.dinv,
        a.rhs, b.p0, b.p1, a.y, b.states, b.col_part, b.err);
}

template <int MODE>
void launch_apply_prec(MfBatch &b, int prec, const ApplyArgs &a) {
    switch (prec) {
        case MG_MIXED_TF32: launch_apply<MG_MIXED_TF32, MODE>(b, a); break;
        case MG_MIXED_BF16: launch_apply<MG_MIXED_BF16, MODE>(b, a); break;
        case MG_MIXED_TF32X3: launch_apply<MG_MIXED_TF32X3, MODE>(b, a); break;
        default: launch_apply<MG_MIXED_BF16X3, MODE>(b, a); break;
    }
}

// level operator of the multigrid (MODE 2: y = rhs - A x, MODE 3: y = A x) on
// level l: the factored CUDA-core operator (fac) or the tensor-core column
// operator in precision prec (x is the vector of map in_slot there)
// the factored kernel's tensor map of a batch vector
int fac_map_of(const MfBatch &b, const float *v) {
    if (v == b.mx) return kFMapMx;
    if (v == b.md) return kFMapMd;
    if (v == b.my) return kFMapMy;
    if (v == b.mb) return kFMapMb;
    if (v == b.r) return kFMapR;
    if (v == b.mr) return kFMapMr;
    return -1;
}

template <int MODE>
void launch_fac(MfBatch &b, int lo, int hi, int sel, const FacArgs &a) {
    if (a.in_map < 0 || ((MODE == 2 || MODE == 4) && a.b_map < 0)) {
        b.enqueue_error = MG_EINVAL;  // reported by the caller of the enqueue
        return;
    }
    if (hi <= lo) return;
    const int grid = std::max(1, std::min(hi - lo, b.fac_grid));
    launch_pdl(mf_fac_kernel<MODE>, grid, kFThreads, fac_smem(MODE), b.stream, b.probs, b.fac_tiles, lo, hi, sel, b.fac2,
                                                                      b.fac_maps, b.states, a, b.err);
}

template <int MODE>
void launch_level_op(MfBatch &b, bool fac, int prec, int l, int in_slot, const float *x, const float *rhs,
                     float *y, int sel) {
    if (fac) {
        launch_fac<MODE>(b, b.lvl_fac_lo[l], b.lvl_fac_hi[l], sel,
                         FacArgs{fac_map_of(b, x), rhs ? fac_map_of(b, rhs) : -1, y, nullptr, nullptr, 0.0f, 0.0f,
                                 0.0f, 0});
    } else {
        ApplyArgs a{b.lvl_col_lo[l], b.lvl_col_hi[l], in_slot, 0, rhs, y, sel};
        launch_apply_prec<MODE>(b, prec, a);
    }
}

// CG step on the level-0 bricks (z from map in_slot)
void launch_cg_apply(MfBatch &b, int prec, int in_slot, int parity) {
    ApplyArgs a{b.lvl_col_lo[0], b.lvl_col_hi[0], in_slot, parity, nullptr, b.q};
    launch_apply_prec<1>(b, prec, a);
}

template <int PREC>
int set_apply_attrs() {
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_col_kernel<PREC, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kColSmem));
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_col_kernel<PREC, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kColSmem));
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_col_kernel<PREC, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, kColSmem));
    // all of the unified L1/shared storage as shared memory: three CTAs per SM
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_col_kernel<PREC, 1>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_col_kernel<PREC, 2>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_col_kernel<PREC, 3>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    return MG_OK;
}

int configure_kernels() {
    static bool done = false;
    if (done) return MG_OK;
    MG_TRY(set_apply_attrs<MG_MIXED_TF32>());
    MG_TRY(set_apply_attrs<MG_MIXED_BF16>());
    MG_TRY(set_apply_attrs<MG_MIXED_TF32X3>());
    MG_TRY(set_apply_attrs<MG_MIXED_BF16X3>());
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_residual64_kernel,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, kResidSmem));
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_fac_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, fac_smem(2)));
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_fac_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, fac_smem(3)));
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_fac_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, fac_smem(4)));
    MG_CUDA_TRY(cudaFuncSetAttribute(mf_fac_kernel<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, fac_smem(5)));
    MG_CUDA_TRY(cudaFuncSetAttribute(mg_bottom_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kBottomSmemMax));
    MG_CUDA_TRY(cudaFuncSetAttribute(mg_coarse_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kCoarseInvSmem));
    MG_CUDA_TRY(cudaFuncSetAttribute(mg_bottom_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    MG_CUDA_TRY(cudaFuncSetAttribute(mg_bottom_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kBottomSmemMax));
    done = true;
    return MG_OK;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_fn(EncodeTiledFn *fn) {
    static EncodeTiledFn cached = nullptr;
    if (!cached) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        MG_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                     cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !p) {
            set_error("cuTensorMapEncodeTiled unavailable");
            return MG_ECUDA;
        }
        cached = reinterpret_cast<EncodeTiledFn>(p);
    }
    *fn = cached;
    return MG_OK;
}

int make_map(EncodeTiledFn fn, CUtensorMap *m, void *base, uint64_t d0, uint64_t d1, uint64_t d2,
             uint64_t stride1_bytes, uint64_t stride2_bytes, uint32_t b0, uint32_t b1, uint32_t b2) {
    cuuint64_t dims[3] = {d0, d1, d2};
    cuuint64_t strides[2] = {stride1_bytes, stride2_bytes};
    cuuint32_t box[3] = {b0, b1, b2};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return MG_ECUDA;
    }
    return MG_OK;
}

int read_states(MfBatch &b) {
    MG_CUDA_TRY(cudaMemcpyAsync(b.states_host, b.states, b.n_probs * sizeof(MfState),
                                cudaMemcpyDeviceToHost, b.stream));
    MG_CUDA_TRY(cudaStreamSynchronize(b.stream));
    int herr = 0;
    MG_CUDA_TRY(cudaMemcpy(&herr, b.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
        set_error("tensor-core pipeline wait exceeded its bound (error flag %d)", herr);
        return MG_ETIMEDOUT;
    }
    return MG_OK;
}

void launch_update(MfBatch &b, float *pnew, bool mg) {
    const int n0 = b.lvl_chunk_hi[0];
    launch_pdl(mf_update_kernel, std::max(1, std::min(n0, b.vec_grid)), kThreads, 0, b.stream, 
        b.chunks, n0, b.probs, b.x, b.r, b.z, pnew, b.q, b.dinv, b.states, b.chunk_part, mg ? 1 : 0);
}

int compute_diag(MfBatch &b) {
    int64_t maxpad = 1;
    for (const MfProblem &P : b.h_probs) maxpad = std::max(maxpad, P.n_pad);
    dim3 grid(std::max(1u, std::min(blocks_for(maxpad, 256), 4096u)), b.n_probs);
    mf_diag_kernel<<<grid, 256, 0, b.stream>>>(b.probs, nullptr, b.E32, b.node_fix, b.K0, b.dinv);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    return MG_OK;  // the operator-only paths need no coarse inverse; activation forms it
}

// Jacobi inverse of the listed level-0 problems and all their coarse levels, and
// the inverse of the coarsest grid of their direct chains; nothing waits on the host
int compute_diag_list(MfBatch &b, const std::vector<int> &level0) {
    std::vector<int> list, inv;
    int64_t maxpad = 1;
    for (int i : level0)
        for (int q = i; q >= 0; q = b.h_probs[q].coarse) {
            list.push_back(q);
            maxpad = std::max(maxpad, b.h_probs[q].n_pad);
        }
    if (list.empty()) return MG_OK;
    for (size_t h = 0; h < b.h_heads.size(); h++)
        if (b.h_coarse_off[h] >= 0 && std::find(level0.begin(), level0.end(), b.h_head_root[h]) != level0.end())
            inv.push_back((int)h);
    // the pinned staging buffer: the previous call's copy must have read it
    if (b.stage_pending) MG_CUDA_TRY(cudaEventSynchronize(b.stage_ev));
    memcpy(b.stage_host, list.data(), list.size() * sizeof(int));
    memcpy(b.stage_host + list.size(), inv.data(), inv.size() * sizeof(int));
    MG_CUDA_TRY(cudaMemcpyAsync(b.diag_list, b.stage_host, (list.size() + inv.size()) * sizeof(int),
                                cudaMemcpyHostToDevice, b.stream));
    MG_CUDA_TRY(cudaEventRecord(b.stage_ev, b.stream));
    b.stage_pending = true;
    dim3 grid(std::max(1u, std::min(blocks_for(maxpad, 256), 4096u)), (unsigned)list.size());
    mf_diag_kernel<<<grid, 256, 0, b.stream>>>(b.probs, b.diag_list, b.E32, b.node_fix, b.K0, b.dinv);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    if (!inv.empty()) {
        mg_coarse_inverse_kernel<<<(unsigned)inv.size(), kCoarseInvThreads, kCoarseInvSmem, b.stream>>>(
            b.probs, b.heads, b.diag_list + list.size(), b.E32, b.dinv, b.K0, b.coarse_off, b.coarse_inv,
            b.coarse_ok);
        MG_CUDA_TRY(cudaGetLastError());
        count_launches(1);
    }
    return MG_OK;
}

}  // namespace

// ----------------------------------------------------------------------- host
void hex8_box_stiffness(double hx, double hy, double hz, double nu, double K[576]) {
    // same quadrature as the FP64 element kernel: 2x2x2 Gauss, E = 1
    const double gp = 0.57735026918962576451;
    const double lam = nu / (1.0 - nu - 2.0 * nu * nu), mu = 1.0 / (2.0 * (1.0 + nu));
    double S[8][8][9];
    memset(S, 0, sizeof(S));
    for (int q = 0; q < 8; q++) {
        const double xi = (q & 1) ? gp : -gp, eta = (q >> 1 & 1) ? gp : -gp, zeta = (q >> 2 & 1) ? gp : -gp;
        const double w = (hx * hy * hz) / 8.0;  // det J, unit weights
        double g[8][3];
        for (int a = 0; a < 8; a++) {
            int dx, dy, dz;
            corner_bits(a, dx, dy, dz);
            const double sx = dx ? 1 : -1, sy = dy ? 1 : -1, sz = dz ? 1 : -1;
            const double fx = 0.5 * (1 + sx * xi), fy = 0.5 * (1 + sy * eta), fz = 0.5 * (1 + sz * zeta);
            g[a][0] = 0.5 * sx * fy * fz * (2.0 / hx);
            g[a][1] = 0.5 * sy * fx * fz * (2.0 / hy);
            g[a][2] = 0.5 * sz * fx * fy * (2.0 / hz);
        }
        for (int a = 0; a < 8; a++)
            for (int b = 0; b < 8; b++)
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < 3; j++) S[a][b][i * 3 + j] += w * g[a][i] * g[b][j];
    }
    for (int a = 0; a < 8; a++)
        for (int b = 0; b < 8; b++) {
            const double *s = S[a][b];
            const double tr = s[0] + s[4] + s[8];
            for (int i = 0; i < 3; i++)
                for (int j = 0; j < 3; j++)
                    K[(3 * a + i) * 24 + 3 * b + j] = lam * s[i * 3 + j] + mu * s[j * 3 + i] + (i == j ? mu * tr : 0.0);
        }
}

// shared-memory layout of the cluster bottom kernel for clusters of cs CTAs: per
// chain its level table (nodes per CTA, offsets of D^-1, E and the CTA's slabs);
// returns the dynamic shared memory (bytes) of the largest chain
int64_t cluster_layout(const MfBatch &b, int cs, std::vector<ClusterChain> &chains) {
    chains.assign(b.h_heads.size(), ClusterChain{});
    int64_t most = 0;
    for (size_t h = 0; h < b.h_heads.size(); h++) {
        ClusterChain &ch = chains[h];
        ch.root = b.h_head_root[h];
        int m = 0;
        int64_t stage = 0;
        for (int t = b.h_heads[h]; t >= 0 && m < kBottomMaxLevels; t = b.h_probs[t].coarse, m++) {
            const MfProblem &T = b.h_probs[t];
            ClusterLevel &L = ch.L[m];
            L.NX = T.NX; L.NY = T.NY; L.NZ = T.NZ;
            L.nx = T.nx; L.ny = T.ny; L.nz = T.nz;
            L.pitch = T.pitch; L.pitch_e = T.pitch_e;
            L.dof_off = T.dof_off; L.elem_off = T.elem_off;
            const int nn = T.NX * T.NY * T.NZ, H = T.NX * T.NY + T.NX + 1;
            L.chunk = (nn + cs - 1) / cs;
            L.NXY = T.NX * T.NY;
            L.rNX = 1.0f / (float)T.NX;
            L.rNXY = 1.0f / (float)L.NXY;
            L.rchunk = 1.0f / (float)L.chunk;
            // the device divides by one rounded product: check it for every node
            auto fdiv = [](int n, float r) { return (int)(((float)n + 0.5f) * r); };
            for (int n = 0; n < nn; n++)
                if (fdiv(n, L.rNXY) != n / L.NXY || fdiv(n, L.rchunk) != n / L.chunk ||
                    (n < L.NXY && fdiv(n, L.rNX) != n / T.NX))
                    return -1;
            for (int r = 0; r < cs; r++) {
                const int n0 = r * L.chunk, n1 = std::min(nn, n0 + L.chunk);
                if (n0 < n1) stage = std::max<int64_t>(stage, 3LL * (std::min(nn - 1, n1 - 1 + H) - std::max(0, n0 - H) + 1));
            }
        }
        ch.m = m;
        int64_t off = kClusterK0;
        ch.s_stage = (int)off;
        off += (stage + 3) / 4 * 4;
        for (int l = 0; l < m; l++) {
            ClusterLevel &L = ch.L[l];
            const int64_t nn = (int64_t)L.NX * L.NY * L.NZ, ne = (int64_t)L.nx * L.ny * L.nz;
            L.s_dinv = (int)off;
            off += (3 * nn + 3) / 4 * 4;
            L.s_E = (int)off;
            off += (ne + 3) / 4 * 4;
            L.s_vec = (int)off;
            off += 15LL * L.chunk;
        }
        most = std::max(most, off * 4);
    }
    return most;
}

int mf_batch_init(MfBatch &b, const std::vector<MfProblem> &shapes, double hx, double hy,
                  double hz, double nu, cudaStream_t stream, int max_levels, bool bottom_cluster) {
    MG_TRY(configure_kernels());
    EncodeTiledFn enc = nullptr;
    MG_TRY(encode_fn(&enc));
    int dev = 0, sms = 0;
    MG_CUDA_TRY(cudaGetDevice(&dev));
    MG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    b.stream = stream;
    b.hx = hx; b.hy = hy; b.hz = hz; b.nu = nu;
    // level 0: the designs; then every design's coarse levels, ordered by level
    b.n_fine = (int)shapes.size();
    b.h_probs.clear();
    for (size_t i = 0; i < shapes.size(); i++) {
        MfProblem P = shapes[i];
        P.level = 0;
        P.root = (int)i;
        P.coarse = -1;
        P.fine = -1;
        b.h_probs.push_back(P);
    }
    b.lvl_prob_lo.assign(1, 0);
    b.lvl_prob_hi.assign(1, b.n_fine);
    for (int lev = 1; lev < std::max(1, std::min(max_levels, kMaxLevels)); lev++) {
        const int lo = b.lvl_prob_lo.back(), hi = b.lvl_prob_hi.back();
        const int start = (int)b.h_probs.size();
        for (int f = lo; f < hi; f++) {
            const MfProblem F = b.h_probs[f];
            if (F.nx % 2 || F.ny % 2 || F.nz % 2 || F.nx < 4 || F.ny < 4 || F.nz < 4) continue;
            MfProblem C{};
            C.nx = F.nx / 2; C.ny = F.ny / 2; C.nz = F.nz / 2;
            C.level = lev;
            C.root = F.root;
            C.fine = f;
            C.coarse = -1;
            // a load case sharing its design's moduli shares the coarse moduli too
            C.share_elems = (F.share_elems >= 0) ? b.h_probs[F.share_elems].coarse : -1;
            b.h_probs[f].coarse = (int)b.h_probs.size();
            b.h_probs.push_back(C);
        }
        if ((int)b.h_probs.size() == start) break;
        b.lvl_prob_lo.push_back(start);
        b.lvl_prob_hi.push_back((int)b.h_probs.size());
    }
    b.n_levels = (int)b.lvl_prob_lo.size();
    b.n_probs = (int)b.h_probs.size();
    int64_t dof = 0, el = 0, nd = 0;
    int nb = 0, nc = 0;
    b.h_bricks.clear();
    b.h_chunks.clear();
    b.h_cols.clear();
    b.h_fac_tiles.clear();
    std::vector<int64_t> level_count(b.n_levels + 1, 0);  // problems per multigrid level
    for (const MfProblem &P : b.h_probs) level_count[P.level]++;
    for (size_t pi = 0; pi < b.h_probs.size(); pi++) {
        MfProblem &P = b.h_probs[pi];
        if (P.nx <= 0 || P.ny <= 0 || P.nz <= 0 || P.nx >= 32767 * kBN || P.ny >= 32767 * kBN ||
            P.nz >= 32767 * kBN) {
            set_error("bad grid %dx%dx%d", P.nx, P.ny, P.nz);
            return MG_EINVAL;
        }
        P.NX = P.nx + 1; P.NY = P.ny + 1; P.NZ = P.nz + 1;
        P.pitch = (3 * P.NX + 3) / 4 * 4;
        P.pitch_e = (P.nx + 3) / 4 * 4;
        P.n_dofs = (int64_t)P.NX * P.NY * P.NZ * 3;
        P.n_pad = (int64_t)P.pitch * P.NY * P.NZ;
        if (P.share_elems >= 0 && P.share_elems < (int)pi) {
            const MfProblem &S = b.h_probs[P.share_elems];
            if (S.nx != P.nx || S.ny != P.ny || S.nz != P.nz) {
                set_error("shared element tables need equal grids");
                return MG_EINVAL;
            }
            P.elem_off = S.elem_off;
        } else {
            P.share_elems = -1;
            P.elem_off = el;
            el += (int64_t)P.pitch_e * P.ny * P.nz;
        }
        P.dof_off = dof;
        P.node_off = nd;
        dof += P.n_pad;
        nd += (int64_t)P.NX * P.NY * P.NZ;
        const int bx = (P.NX + kBN - 1) / kBN, by = (P.NY + kBN - 1) / kBN, bz = (P.NZ + kBN - 1) / kBN;
        P.brick_begin = nb;
        P.brick_count = bx * by * bz;
        for (int k = 0; k < bz; k++)
            for (int j = 0; j < by; j++)
                for (int i = 0; i < bx; i++)
                    b.h_bricks.push_back(MfBrick{(int)pi, (int16_t)i, (int16_t)j, (int16_t)k, 0});
        nb += P.brick_count;
        // columns of the tensor-core operator: as deep as one wave of resident
        // columns allows (the level's problems share the 3 x SM slots), 4 to kCZ
        // node planes; a second, partial wave would double the launch's time
        const int cx = (P.NX + kCX - 1) / kCX, cy = (P.NY + kCY - 1) / kCY;
        const int64_t slots = kColCtas * (int64_t)sms;
        const int64_t col_per = std::max<int64_t>(1, slots / ((int64_t)cx * cy * level_count[P.level]));
        P.col_z = (int)std::min<int64_t>(kCZ, std::max<int64_t>(4, (P.NZ + col_per - 1) / col_per));
        const int cz = (P.NZ + P.col_z - 1) / P.col_z;
        P.col_begin = (int)b.h_cols.size();
        P.col_count = cx * cy * cz;
        for (int k = 0; k < cz; k++)
            for (int j = 0; j < cy; j++)
                for (int i = 0; i < cx; i++)
                    b.h_cols.push_back(MfCol{(int)pi, (int16_t)i, (int16_t)j, (int16_t)k, 0});
        // tiles of the factored operator: kFNX x kFNY owned nodes, fac_z node
        // planes (kFMinZ .. kFMaxZ): as deep as one wave of resident tiles allows
        {
            const int tx = (P.NX + kFNX - 1) / kFNX, ty = (P.NY + kFNY - 1) / kFNY;
            const int64_t fac_slots = 2 * (int64_t)sms;
            const int64_t per_col = std::max<int64_t>(1, fac_slots / ((int64_t)tx * ty * level_count[P.level]));
            P.fac_z = (int)std::min<int64_t>(kFMaxZ, std::max<int64_t>(kFMinZ, (P.NZ + per_col - 1) / per_col));
            const int tz = (P.NZ + P.fac_z - 1) / P.fac_z;
            P.fac_begin = (int)b.h_fac_tiles.size();
            P.fac_count = tx * ty * tz;
            for (int k = 0; k < tz; k++)
                for (int j = 0; j < ty; j++)
                    for (int i = 0; i < tx; i++)
                        b.h_fac_tiles.push_back(MfCol{(int)pi, (int16_t)i, (int16_t)j, (int16_t)k, 0});
        }
        P.chunk_begin = nc;
        P.chunk_count = (int)((P.n_pad + kChunk - 1) / kChunk);
        for (int c = 0; c < P.chunk_count; c++) {
            MfChunkDesc C;
            C.prob = (int)pi;
            C.pad = 0;
            C.begin = P.dof_off + (int64_t)c * kChunk;
            C.end = std::min(P.dof_off + P.n_pad, C.begin + kChunk);
            b.h_chunks.push_back(C);
        }
        nc += P.chunk_count;
    }
    b.n_bricks = nb;
    b.n_chunks = nc;
    b.n_cols = (int)b.h_cols.size();
    b.lvl_brick_lo.clear(); b.lvl_brick_hi.clear(); b.lvl_chunk_lo.clear(); b.lvl_chunk_hi.clear();
    b.lvl_col_lo.clear(); b.lvl_col_hi.clear();
    b.lvl_fac_lo.clear(); b.lvl_fac_hi.clear();
    for (int l = 0; l < b.n_levels; l++) {
        const MfProblem &A = b.h_probs[b.lvl_prob_lo[l]], &Z = b.h_probs[b.lvl_prob_hi[l] - 1];
        b.lvl_brick_lo.push_back(A.brick_begin);
        b.lvl_brick_hi.push_back(Z.brick_begin + Z.brick_count);
        b.lvl_col_lo.push_back(A.col_begin);
        b.lvl_col_hi.push_back(Z.col_begin + Z.col_count);
        b.lvl_fac_lo.push_back(A.fac_begin);
        b.lvl_fac_hi.push_back(Z.fac_begin + Z.fac_count);
        b.lvl_chunk_lo.push_back(A.chunk_begin);
        b.lvl_chunk_hi.push_back(Z.chunk_begin + Z.chunk_count);
    }
    b.n_pad = dof;
    b.n_elem_pad = el;
    b.n_nodes = nd;
    // bottom chains: for every design, the first level below the finest with at
    // most kBottomMaxHeadNodes nodes whose chain (it and all coarser levels) fits
    // the bottom kernel's shared memory; larger levels run level by level on the
    // whole GPU (the one-CTA kernel is bound by one SM's shared-memory pipe there).
    // With a cluster per chain (bottom_cluster: single-design solves), the first
    // level with at most kClusterMaxHeadNodes nodes.
    // (a device on which no cluster of the bottom kernel can be placed falls back
    // to the one-CTA chains)
    int64_t inv_floats = 0;
    for (int attempt = bottom_cluster ? 0 : 1; attempt < 2; attempt++) {
        const bool use_cluster = attempt == 0;
        b.h_heads.clear();
        b.h_head_root.clear();
        b.bottom_smem = 0;
        b.bottom_cluster = 0;
        for (MfProblem &T : b.h_probs) T.bottom = 0;
        for (int r = 0; r < b.n_fine; r++) {
            for (int q = b.h_probs[r].coarse; q >= 0; q = b.h_probs[q].coarse) {
                int64_t floats = 576 + 800, depth = 0;
                for (int t = q; t >= 0; t = b.h_probs[t].coarse, depth++) {
                    const MfProblem &T = b.h_probs[t];
                    // x, b, r, d, y, D^-1 per dof and E per element
                    floats += 18LL * T.NX * T.NY * T.NZ + (int64_t)T.nx * T.ny * T.nz;
                }
                const int64_t bytes = floats * 4;
                const MfProblem &Hd = b.h_probs[q];
                const int64_t head_nodes = (int64_t)Hd.NX * Hd.NY * Hd.NZ;
                const bool fits = use_cluster ? head_nodes <= kClusterMaxHeadNodes
                                              : bytes <= kBottomSmemMax && head_nodes <= kBottomMaxHeadNodes;
                if (depth <= kBottomMaxLevels && fits) {
                    b.h_heads.push_back(q);
                    b.h_head_root.push_back(r);
                    b.bottom_smem = use_cluster ? (576 + 800) * 4 : std::max(b.bottom_smem, (int)bytes);
                    for (int t = q; t >= 0; t = b.h_probs[t].coarse) b.h_probs[t].bottom = 1;
                    break;
                }
            }
        }
        // direct coarse solves: the chains whose coarsest grid is small enough and
        // whose inverse fits the bottom kernel's shared memory beside the levels
        {
            inv_floats = 0;
            b.h_coarse_off.assign(b.h_heads.size(), -1);
            for (size_t h = 0; h < b.h_heads.size(); h++) {
                int64_t floats = 576 + 800;
                int c = b.h_heads[h];
                for (int t = c; t >= 0; t = b.h_probs[t].coarse) {
                    const MfProblem &T = b.h_probs[t];
                    floats += 18LL * T.NX * T.NY * T.NZ + (int64_t)T.nx * T.ny * T.nz;
                    c = t;
                }
                const MfProblem &C = b.h_probs[c];
                const int64_t nd = 3LL * C.NX * C.NY * C.NZ;
                if (nd <= kCoarseDirectMax && (use_cluster || (floats + nd * nd) * 4 <= kBottomSmemMax)) {
                    b.h_coarse_off[h] = inv_floats;
                    inv_floats += nd * nd;
                    if (!use_cluster) b.bottom_smem = std::max(b.bottom_smem, (int)((floats + nd * nd) * 4));
                }
            }
        }
        if (!use_cluster || b.h_heads.empty()) break;
        {
            // the largest cluster (16 CTAs: non-portable size) the device can place
            // MASTGPU_BOTTOM_CLUSTER caps the cluster (1, 2, 4, 8 or 16 CTAs): a test knob,
            // the result does not depend on the cluster size
            int cap = kClusterMax;
            if (const char *env = std::getenv("MASTGPU_BOTTOM_CLUSTER")) cap = std::max(1, std::min(kClusterMax, std::atoi(env)));
            int first = 1;
            while (first * 2 <= cap) first *= 2;
            for (int cs = first; cs >= 1 && !b.bottom_cluster; cs /= 2) {
                std::vector<ClusterChain> chains;
                const int64_t smem = cluster_layout(b, cs, chains);
                if (smem < 0 || smem > kBottomSmemMax) continue;
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(cs);
                cfg.blockDim = dim3(kClusterThreads);
                cfg.dynamicSmemBytes = smem;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = (unsigned)cs;
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                int n = 0;
                if (cudaOccupancyMaxActiveClusters(&n, mg_bottom_cluster_kernel, &cfg) == cudaSuccess && n >= 1) {
                    b.bottom_cluster = cs;
                    b.bottom_smem = (int)smem;
                    b.h_cl_chains.swap(chains);
                }
                else
                    cudaGetLastError();  // clear the failed query
            }
        }
        if (b.bottom_cluster) break;
    }
    MG_TRY(dev_alloc_n(&b.coarse_off, std::max<size_t>(1, b.h_coarse_off.size())));
    MG_TRY(dev_alloc_n(&b.coarse_inv, (size_t)std::max<int64_t>(1, inv_floats)));
    MG_TRY(dev_alloc_n(&b.coarse_ok, std::max<size_t>(1, b.h_coarse_off.size())));
    b.apply_grid = std::max(1, std::min(nb, 2 * sms));  // FP64 residual: two CTAs per SM
    b.col_grid = std::max(1, std::min(b.n_cols, kColCtas * sms));  // column CTAs per SM
    b.fac_grid = 2 * sms;                                     // two factored-operator CTAs per SM
    b.vec_grid = std::max(1, std::min(nc, 8 * sms));
    MG_TRY(dev_alloc_n(&b.probs, b.h_probs.size()));
    MG_TRY(dev_alloc_n(&b.bricks, b.h_bricks.size()));
    MG_TRY(dev_alloc_n(&b.cols, b.h_cols.size()));
    MG_TRY(dev_alloc_n(&b.col_part, b.h_cols.size()));
    MG_TRY(dev_alloc_n(&b.fac_tiles, std::max<size_t>(1, b.h_fac_tiles.size())));
    MG_TRY(dev_alloc_n(&b.Bop2, 4096));
    MG_TRY(dev_alloc_n(&b.chunks, b.h_chunks.size()));
    MG_TRY(dev_alloc_n(&b.states, (size_t)b.n_probs));
    MG_TRY(dev_alloc_n(&b.tmaps, (size_t)b.n_probs * kMapsPerProblem));
    MG_TRY(dev_alloc_n(&b.fac_maps, (size_t)b.n_probs * kFacMaps));
    MG_CUDA_TRY(cudaMallocHost(reinterpret_cast<void **>(&b.states_host), b.n_probs * sizeof(MfState)));
    MG_TRY(dev_alloc_n(&b.E32, (size_t)el + 4));
    MG_TRY(dev_alloc_n(&b.Edf, (size_t)el + 4));
    MG_TRY(dev_alloc_n(&b.dE64, (size_t)el + 4));
    MG_TRY(dev_alloc_n(&b.node_fix, (size_t)nd));
    float **f32s[] = {&b.x, &b.r, &b.z, &b.p0, &b.p1, &b.q, &b.dinv, &b.xdbg,
                      &b.mb, &b.mx, &b.md, &b.my, &b.mr};
    for (float **v : f32s) MG_TRY(dev_alloc_n(v, (size_t)dof));
    MG_TRY(dev_alloc_n(&b.u64, (size_t)dof));
    MG_TRY(dev_alloc_n(&b.r64, (size_t)dof));
    MG_TRY(dev_alloc_n(&b.f64, (size_t)dof));
    MG_TRY(dev_alloc_n(&b.brick_part, (size_t)2 * nb));  // operator partials | ||f||^2 partials
    MG_TRY(dev_alloc_n(&b.chunk_part, (size_t)2 * nc));
    MG_TRY(dev_alloc_n(&b.err, 1));
    MG_TRY(dev_alloc_n(&b.diag_list, (size_t)b.n_probs + b.h_heads.size()));
    MG_TRY(dev_alloc_n(&b.sens_offs, (size_t)std::max(1, b.n_fine)));
    MG_CUDA_TRY(cudaMallocHost(&b.sens_offs_host, (size_t)std::max(1, b.n_fine) * sizeof(int64_t)));
    MG_CUDA_TRY(cudaMallocHost(&b.stage_host, ((size_t)b.n_probs + b.h_heads.size()) * sizeof(int)));
    MG_CUDA_TRY(cudaEventCreateWithFlags(&b.stage_ev, cudaEventDisableTiming));
    MG_TRY(dev_alloc_n(&b.heads, std::max<size_t>(1, b.h_heads.size())));
    MG_TRY(dev_alloc_n(&b.K0, 576));
    double K0[576];
    hex8_box_stiffness(hx, hy, hz, nu, K0);
    if (!hex8_factored_build(K0, b.fac64, b.fac32)) return MG_EINVAL;
    for (int k = 0; k < kFacN; k++) b.facdf.v[k] = dfloat_of(b.fac64.v[k]);
    for (int k = 0; k < kFacN; k++) b.fac2.v[k] = make_float2(b.fac32.v[k], b.fac32.v[k]);
    // Gershgorin bound of D^-1 A: every assembled row is a positive combination
    // of K0 rows, so max_i sum_j |K0_ij| / K0_ii bounds it on every level
    b.cheb_lmax = 0.0;
    for (int i = 0; i < 24; i++) {
        double sabs = 0.0;
        for (int j = 0; j < 24; j++) sabs += fabs(K0[i * 24 + j]);
        b.cheb_lmax = std::max(b.cheb_lmax, sabs / K0[i * 24 + i]);
    }
    // tensor maps: z, p0, p1, E, debug x per problem
    std::vector<CUtensorMap> maps(b.n_probs * kMapsPerProblem);
    for (int pi = 0; pi < b.n_probs; pi++) {
        const MfProblem &P = b.h_probs[pi];
        float *vecs[5] = {b.z, b.p0, b.p1, b.mx, b.md};
        const int slot[5] = {0, 1, 2, 4, 5};
        // column operator: one node plane {32 floats, 17 rows} / element plane {12, 16}
        for (int k = 0; k < 5; k++)
            MG_TRY(make_map(enc, &maps[pi * kMapsPerProblem + slot[k]], vecs[k] + P.dof_off,
                            3 * (uint64_t)P.NX, P.NY, P.NZ, (uint64_t)P.pitch * 4,
                            (uint64_t)P.pitch * P.NY * 4, kCRawX, kCPY, 1));
        MG_TRY(make_map(enc, &maps[pi * kMapsPerProblem + 3], b.E32 + P.elem_off, P.nx, P.ny, P.nz,
                        (uint64_t)P.pitch_e * 4, (uint64_t)P.pitch_e * P.ny * 4, 12, 16, 1));
    }
    // factored level operator: node planes {104 floats, 17 rows}, moduli planes {36, 16}
    std::vector<CUtensorMap> fmaps((size_t)b.n_probs * kFacMaps);
    for (int pi = 0; pi < b.n_probs; pi++) {
        const MfProblem &P = b.h_probs[pi];
        float *vecs[kFMapE] = {b.mx, b.md, b.my, b.mb, b.r, b.dinv, b.mr};
        for (int k = 0; k < kFMapE; k++)
            MG_TRY(make_map(enc, &fmaps[(size_t)pi * kFacMaps + k], vecs[k] + P.dof_off, 3 * (uint64_t)P.NX, P.NY,
                            P.NZ, (uint64_t)P.pitch * 4, (uint64_t)P.pitch * P.NY * 4, kFBoxX, kFPY, 1));
        MG_TRY(make_map(enc, &fmaps[(size_t)pi * kFacMaps + kFMapE], b.E32 + P.elem_off, P.nx, P.ny, P.nz,
                        (uint64_t)P.pitch_e * 4, (uint64_t)P.pitch_e * P.ny * 4, kFBoxE, kFEY, 1));
    }
    cudaStream_t s = b.stream;
    MG_CUDA_TRY(cudaMemcpyAsync(b.tmaps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, s));
    MG_CUDA_TRY(cudaMemcpyAsync(b.fac_maps, fmaps.data(), fmaps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, s));
    MG_CUDA_TRY(cudaMemcpyAsync(b.probs, b.h_probs.data(), b.h_probs.size() * sizeof(MfProblem), cudaMemcpyHostToDevice, s));
    MG_CUDA_TRY(cudaMemcpyAsync(b.bricks, b.h_bricks.data(), b.h_bricks.size() * sizeof(MfBrick), cudaMemcpyHostToDevice, s));
    MG_CUDA_TRY(cudaMemcpyAsync(b.cols, b.h_cols.data(), b.h_cols.size() * sizeof(MfCol), cudaMemcpyHostToDevice, s));
    if (!b.h_fac_tiles.empty())
        MG_CUDA_TRY(cudaMemcpyAsync(b.fac_tiles, b.h_fac_tiles.data(), b.h_fac_tiles.size() * sizeof(MfCol),
                                    cudaMemcpyHostToDevice, s));
    {
        std::vector<uint32_t> bop2;
        pack_b_columns(K0, bop2);
        MG_CUDA_TRY(cudaMemcpyAsync(b.Bop2, bop2.data(), bop2.size() * 4, cudaMemcpyHostToDevice, s));
        MG_CUDA_TRY(cudaStreamSynchronize(s));  // bop2 is a host temporary
    }
    MG_CUDA_TRY(cudaMemcpyAsync(b.chunks, b.h_chunks.data(), b.h_chunks.size() * sizeof(MfChunkDesc), cudaMemcpyHostToDevice, s));
    MG_CUDA_TRY(cudaMemcpyAsync(b.K0, K0, 576 * 8, cudaMemcpyHostToDevice, s));
    if (b.bottom_cluster) {
        // K0 and its regrouped copy in FP32 (as mg_bottom_kernel forms them), the chains' level tables
        std::vector<float> k0f(kClusterK0);
        for (int i = 0; i < 576; i++) k0f[i] = (float)K0[i];
        for (int i = 0; i < 800; i++) {
            const int a = i / 100, t = i % 100, bc = t / 12, q = t % 12, r = q / 3, c = q % 3;
            k0f[576 + i] = (t < 96 && q < 9) ? (float)K0[(3 * a + r) * 24 + 3 * bc + c] : 0.0f;
        }
        MG_TRY(dev_alloc_n(&b.cl_k0, (size_t)kClusterK0));
        MG_TRY(dev_alloc_n(&b.cl_chains, b.h_cl_chains.size()));
        MG_CUDA_TRY(cudaMemcpyAsync(b.cl_k0, k0f.data(), k0f.size() * 4, cudaMemcpyHostToDevice, s));
        MG_CUDA_TRY(cudaMemcpyAsync(b.cl_chains, b.h_cl_chains.data(), b.h_cl_chains.size() * sizeof(ClusterChain),
                                    cudaMemcpyHostToDevice, s));
        MG_CUDA_TRY(cudaStreamSynchronize(s));  // k0f is a host temporary
    }
    if (!b.h_coarse_off.empty()) {
        MG_CUDA_TRY(cudaMemcpyAsync(b.coarse_off, b.h_coarse_off.data(), b.h_coarse_off.size() * sizeof(int64_t),
                                    cudaMemcpyHostToDevice, s));
        MG_CUDA_TRY(cudaMemsetAsync(b.coarse_ok, 0, b.h_coarse_off.size() * sizeof(int), s));
    }
    if (!b.h_heads.empty())
        MG_CUDA_TRY(cudaMemcpyAsync(b.heads, b.h_heads.data(), b.h_heads.size() * sizeof(int),
                                    cudaMemcpyHostToDevice, s));
    MG_CUDA_TRY(cudaMemsetAsync(b.states, 0, b.n_probs * sizeof(MfState), s));
    MG_CUDA_TRY(cudaMemsetAsync(b.err, 0, sizeof(int), s));
    MG_CUDA_TRY(cudaMemsetAsync(b.u64, 0, dof * 8, s));
    MG_CUDA_TRY(cudaMemsetAsync(b.r64, 0, dof * 8, s));
    MG_CUDA_TRY(cudaMemsetAsync(b.f64, 0, dof * 8, s));
    MG_CUDA_TRY(cudaMemsetAsync(b.node_fix, 0, nd, s));
    MG_CUDA_TRY(cudaMemsetAsync(b.E32, 0, (el + 4) * 4, s));
    MG_CUDA_TRY(cudaMemsetAsync(b.Edf, 0, (el + 4) * sizeof(dfloat), s));
    MG_CUDA_TRY(cudaMemsetAsync(b.dE64, 0, (el + 4) * 8, s));
    float *zero_vecs[] = {b.x, b.r, b.z, b.p0, b.p1, b.q, b.dinv, b.xdbg, b.mb, b.mx, b.md, b.my, b.mr};
    for (float *v : zero_vecs) MG_CUDA_TRY(cudaMemsetAsync(v, 0, dof * 4, s));
    MG_CUDA_TRY(cudaStreamSynchronize(s));
    return MG_OK;
}

void mf_batch_free(MfBatch &b) {
    if (b.stream) cudaStreamSynchronize(b.stream);
    if (b.graph) cudaGraphExecDestroy(b.graph);
    void *ptrs[] = {b.probs, b.bricks, b.chunks, b.states, b.tmaps, b.E32, b.Edf, b.dE64,
                    b.node_fix, b.x, b.r, b.z, b.p0, b.p1, b.q, b.dinv, b.xdbg, b.u64, b.r64,
                    b.f64, b.brick_part, b.chunk_part, b.err, b.K0, b.mb, b.mx, b.md,
                    b.my, b.mr, b.diag_list, b.heads, b.cols, b.col_part, b.Bop2, b.fac_tiles, b.fac_maps,
                    b.coarse_off, b.coarse_inv, b.coarse_ok, b.cl_chains, b.cl_k0, b.sens_offs};
    for (void *q : ptrs) dev_free(q);
    if (b.stage_host) cudaFreeHost(b.stage_host);
    if (b.sens_offs_host) cudaFreeHost(b.sens_offs_host);
    if (b.stage_ev) cudaEventDestroy(b.stage_ev);
    if (b.states_host) cudaFreeHost(b.states_host);
    if (b.err_host) cudaFreeHost(b.err_host);
    b = MfBatch();
}

int mf_batch_set_bc(MfBatch &b, int i, const uint8_t *node_fix_host, const double *f_host) {
    if (i < 0 || i >= b.n_probs) return MG_EINVAL;
    const MfProblem &P = b.h_probs[i];
    const int64_t nn = (int64_t)P.NX * P.NY * P.NZ;
    cudaStream_t s = b.stream;
    if (node_fix_host) {
        MG_CUDA_TRY(cudaMemcpyAsync(b.node_fix + P.node_off, node_fix_host, nn, cudaMemcpyHostToDevice, s));
        // coarse levels: a coarse node is constrained where its fine node (2I,2J,2K) is
        std::vector<uint8_t> fine(node_fix_host, node_fix_host + nn), coarse;
        for (int f = i; b.h_probs[f].coarse >= 0; f = b.h_probs[f].coarse) {
            const MfProblem &F = b.h_probs[f], &C = b.h_probs[F.coarse];
            coarse.assign((size_t)C.NX * C.NY * C.NZ, 0);
            for (int K = 0; K < C.NZ; K++)
                for (int J = 0; J < C.NY; J++)
                    for (int I = 0; I < C.NX; I++)
                        coarse[I + (size_t)C.NX * (J + (size_t)C.NY * K)] =
                            fine[2 * I + (size_t)F.NX * (2 * J + (size_t)F.NY * 2 * K)];
            MG_CUDA_TRY(cudaMemcpyAsync(b.node_fix + C.node_off, coarse.data(), coarse.size(),
                                        cudaMemcpyHostToDevice, s));
            MG_CUDA_TRY(cudaStreamSynchronize(s));
            fine.swap(coarse);
        }
    }
    if (f_host) {
        std::vector<double> pad(P.n_pad, 0.0);
        for (int64_t row = 0; row < (int64_t)P.NY * P.NZ; row++)
            memcpy(pad.data() + row * P.pitch, f_host + row * 3 * P.NX, 3 * P.NX * sizeof(double));
        MG_CUDA_TRY(cudaMemcpyAsync(b.f64 + P.dof_off, pad.data(), P.n_pad * 8, cudaMemcpyHostToDevice, s));
        MG_CUDA_TRY(cudaStreamSynchronize(s));  // pad is a host temporary
    }
    if (node_fix_host) MG_CUDA_TRY(cudaStreamSynchronize(s));
    return MG_OK;
}

int mf_batch_set_moduli(MfBatch &b, int i, const double *E_dev, const double *dE_dev) {
    if (i < 0 || i >= b.n_probs) return MG_EINVAL;
    const MfProblem &P = b.h_probs[i];
    const int64_t ne = (int64_t)P.nx * P.ny * P.nz;
    pack_elems_kernel<<<std::min(blocks_for(ne, 256), 4096u), 256, 0, b.stream>>>(
        b.probs, i, E_dev, dE_dev, b.E32, b.Edf, b.dE64);
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(1);
    if (E_dev)
        for (int f = i; b.h_probs[f].coarse >= 0; f = b.h_probs[f].coarse) {
            const int c = b.h_probs[f].coarse;
            const MfProblem &C = b.h_probs[c];
            const int64_t nc = (int64_t)C.nx * C.ny * C.nz;
            dim3 grid(std::min(blocks_for(nc, 256), 4096u), 1);
            mg_coarsen_kernel<<<grid, 256, 0, b.stream>>>(b.probs, c, b.E32);
            MG_CUDA_TRY(cudaGetLastError());
            count_launches(1);
        }
    return MG_OK;
}

int mf_batch_get_u(MfBatch &b, int i, double *u_dev) {
    const MfProblem &P = b.h_probs[i];
    unpack_vec_kernel<<<std::min(blocks_for(P.n_dofs, 256), 4096u), 256, 0, b.stream>>>(
        b.probs, i, b.u64, u_dev, 1);
    MG_CUDA_TRY(cudaGetLastError());
    return MG_OK;
}

int mf_batch_set_u(MfBatch &b, int i, const double *u_dev) {
    const MfProblem &P = b.h_probs[i];
    unpack_vec_kernel<<<std::min(blocks_for(P.n_dofs, 256), 4096u), 256, 0, b.stream>>>(
        b.probs, i, b.u64, const_cast<double *>(u_dev), 0);
    MG_CUDA_TRY(cudaGetLastError());
    return MG_OK;
}

int mf_apply(MfBatch &b, int precision, const double *x_host, double *y_host, int prob) {
    MG_TRY(compute_diag(b));
    const MfProblem &P = b.h_probs[prob];
    std::vector<float> pad(P.n_pad, 0.0f);
    for (int64_t row = 0; row < (int64_t)P.NY * P.NZ; row++)
        for (int64_t k = 0; k < 3 * P.NX; k++) pad[row * P.pitch + k] = (float)x_host[row * 3 * P.NX + k];
    MG_CUDA_TRY(cudaMemcpyAsync(b.mx + P.dof_off, pad.data(), P.n_pad * 4, cudaMemcpyHostToDevice, b.stream));
    MG_CUDA_TRY(cudaMemsetAsync(b.states, 0, b.n_probs * sizeof(MfState), b.stream));
    if (precision == MG_OPERATOR_FACTORED_FP32) {
        launch_fac<3>(b, P.fac_begin, P.fac_begin + P.fac_count, -1,
                      FacArgs{kFMapMx, -1, b.my, nullptr, nullptr, 0.0f, 0.0f, 0.0f, 0});
    } else {
        ApplyArgs a{P.col_begin, P.col_begin + P.col_count, 4, 0, nullptr, b.my};
        launch_apply_prec<3>(b, precision, a);
    }
    MG_CUDA_TRY(cudaGetLastError());
    MG_CUDA_TRY(cudaMemcpyAsync(pad.data(), b.my + P.dof_off, P.n_pad * 4, cudaMemcpyDeviceToHost, b.stream));
    MG_CUDA_TRY(cudaStreamSynchronize(b.stream));
    int herr = 0;
    MG_CUDA_TRY(cudaMemcpy(&herr, b.err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
        set_error("tensor-core pipeline wait exceeded its bound (error flag %d)", herr);
        return MG_ETIMEDOUT;
    }
    for (int64_t row = 0; row < (int64_t)P.NY * P.NZ; row++)
        for (int64_t k = 0; k < 3 * P.NX; k++) y_host[row * 3 * P.NX + k] = pad[row * P.pitch + k];
    return MG_OK;
}

// enqueue `reps` CG-mode operator launches on the level-0 bricks (timing hook; no sync)
int mf_launch_apply(MfBatch &b, int precision, int reps) {
    MG_TRY(compute_diag(b));
    MG_CUDA_TRY(cudaMemsetAsync(b.states, 0, b.n_probs * sizeof(MfState), b.stream));
    // nonzero search direction (zero on Dirichlet dofs) so every launch does the full work
    fill_f32_kernel<<<blocks_for(b.n_pad, 256), 256, 0, b.stream>>>(b.z, b.dinv, 1.0f, b.n_pad);
    if (precision == MG_OPERATOR_FACTORED_FP32) {
        // the multigrid level operator y = A x on level 0 (mx, my)
        fill_f32_kernel<<<blocks_for(b.n_pad, 256), 256, 0, b.stream>>>(b.mx, b.dinv, 1.0f, b.n_pad);
        for (int i = 0; i < reps; i++) launch_level_op<3>(b, true, 0, 0, 4, b.mx, nullptr, b.my, -1);
    } else {
        for (int i = 0; i < reps; i++) launch_cg_apply(b, precision, 0, i & 1);
    }
    MG_CUDA_TRY(cudaGetLastError());
    count_launches(reps + 2);
    return MG_OK;
}

namespace {

// precision of the multigrid smoothers: the single-product form of the family
int mg_precision(int prec) {
    return (prec == MG_MIXED_BF16 || prec == MG_MIXED_BF16X3) ? MG_MIXED_BF16 : MG_MIXED_TF32;
}

// Chebyshev coefficients for degree `deg` on [lmax/30, lmax]
struct Cheb {
    float inv_theta;
    float c1[32], c2[32];
};
Cheb cheb_coeffs(double lmax, int deg) {
    Cheb c{};
    const double lmin = lmax / 30.0, theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    const double sigma = theta / delta;
    double rho = 1.0 / sigma;
    c.inv_theta = (float)(1.0 / theta);
    for (int k = 1; k < deg && k < 32; k++) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        c.c1[k] = (float)(rn * rho);
        c.c2[k] = (float)(2.0 * rn / delta);
        rho = rn;
    }
    return c;
}

// one Chebyshev smoothing pass of degree deg on level l: mx (+)= S(rin), on the
// level's problems selected by sel (see ApplyArgs)
long long enqueue_smooth(MfBatch &b, bool fac, int prec, int l, const float *rin, int x0_zero, int deg,
                         const Cheb &cc, int sel) {
    const int clo = b.lvl_chunk_lo[l], chi = b.lvl_chunk_hi[l];
    const int grid = std::max(1, std::min(chi - clo, b.vec_grid));
    if (fac && deg >= 2) {
        // fused: the first two steps in one launch (direction into md, which is
        // never rin), then one launch per step, the direction alternating md / my
        const int lo = b.lvl_fac_lo[l], hi = b.lvl_fac_hi[l];
        launch_fac<5>(b, lo, hi, sel,
                      FacArgs{fac_map_of(b, rin), kFMapMx, b.md, b.mr, b.mx, cc.c1[1], cc.c2[1], cc.inv_theta, x0_zero});
        float *din = b.md, *dout = b.my;
        long long n = 1;
        for (int k = 2; k < deg; k++) {
            launch_fac<4>(b, lo, hi, sel,
                          FacArgs{fac_map_of(b, din), kFMapMr, dout, b.mr, b.mx, cc.c1[k], cc.c2[k], 0.0f, 0});
            std::swap(din, dout);
            n += 1;
        }
        return n;
    }
    launch_pdl(mg_cheb_first_kernel, grid, kThreads, 0, b.stream, b.chunks, clo, chi, b.probs, b.states, rin,
                                                          b.mr, b.md, b.mx, b.dinv, cc.inv_theta, x0_zero, sel);
    long long n = 1;
    for (int k = 1; k < deg; k++) {
        launch_level_op<3>(b, fac, prec, l, 5, b.md, nullptr, b.my, sel);
        launch_pdl(mg_cheb_next_kernel, grid, kThreads, 0, b.stream, b.chunks, clo, chi, b.probs, b.states, b.my,
                                                             b.mr, b.md, b.mx, b.dinv, cc.c1[k], cc.c2[k], sel);
        n += 2;
    }
    return n;
}

// V-cycle z = M r on every design at once (level-0 rhs = CG residual r, z = mx).
// A problem whose own coarsest grid is level l gets the coarse-grid smoother
// (degree cdeg) there, whatever the depth of the other problems, so that each
// problem's preconditioner does not depend on the batch it is solved in.  The
// small levels of each chain (MfProblem::bottom) are done by one CTA per chain
// (mg_bottom_kernel) between the down and the up sweep.
long long enqueue_vcycle(MfBatch &b, bool fac, int prec, int sdeg, int cdeg) {
    const Cheb cs = cheb_coeffs(b.cheb_lmax, sdeg), cc = cheb_coeffs(b.cheb_lmax, cdeg);
    const int L = b.n_levels;
    auto any_level = [&](int l) {  // some problem of level l is solved level by level
        for (int pi = b.lvl_prob_lo[l]; pi < b.lvl_prob_hi[l]; pi++)
            if (!b.h_probs[pi].bottom) return true;
        return false;
    };
    auto own_coarsest = [&](int l) {  // ... and has no coarser level
        for (int pi = b.lvl_prob_lo[l]; pi < b.lvl_prob_hi[l]; pi++)
            if (!b.h_probs[pi].bottom && b.h_probs[pi].coarse < 0) return true;
        return false;
    };
    long long n = 0;
    for (int l = 0; l < L - 1; l++) {
        if (!any_level(l)) continue;
        const float *rin = (l == 0) ? b.r : b.mb;
        n += enqueue_smooth(b, fac, prec, l, rin, 1, sdeg, cs, 0);
        launch_level_op<2>(b, fac, prec, l, 4, b.mx, rin, b.my, 0);  // my = rin - A mx
        const int clo = b.lvl_prob_lo[l + 1], chi = b.lvl_prob_hi[l + 1];
        int64_t maxnodes = 1;
        for (int pi = clo; pi < chi; pi++)
            maxnodes = std::max<int64_t>(maxnodes, (int64_t)b.h_probs[pi].NX * b.h_probs[pi].NY * b.h_probs[pi].NZ);
        dim3 grid(std::max(1u, std::min(blocks_for(maxnodes, 256), 4096u)), chi - clo);
        launch_pdl(mg_restrict_kernel, grid, 256, 0, b.stream, b.probs, clo, b.states, b.my, b.mb, b.dinv);
        n += 2;
        if (own_coarsest(l)) n += enqueue_smooth(b, fac, prec, l, rin, 1, cdeg, cc, 1);
    }
    if (any_level(L - 1)) n += enqueue_smooth(b, fac, prec, L - 1, L == 1 ? b.r : b.mb, 1, cdeg, cc, -1);
    if (!b.h_heads.empty()) {
        BottomCheb bc{};
        bc.inv_theta_s = cs.inv_theta;
        bc.inv_theta_c = cc.inv_theta;
        for (int k = 0; k < 32; k++) {
            bc.c1s[k] = cs.c1[k]; bc.c2s[k] = cs.c2[k];
            bc.c1c[k] = cc.c1[k]; bc.c2c[k] = cc.c2[k];
        }
        if (b.bottom_cluster)
            launch_cluster_pdl(mg_bottom_cluster_kernel, (unsigned)(b.h_heads.size() * b.bottom_cluster),
                               kClusterThreads, b.bottom_smem, b.bottom_cluster, b.stream, b.cl_chains, b.states,
                               b.E32, b.dinv, b.mb, b.mx, b.cl_k0, bc, sdeg, cdeg, b.coarse_off, b.coarse_inv,
                               b.coarse_ok);
        else
            launch_pdl(mg_bottom_kernel, (unsigned)b.h_heads.size(), kBottomThreads, b.bottom_smem, b.stream,
                b.probs, b.heads, b.states, b.E32, b.dinv, b.mb, b.mx, b.K0, bc, sdeg, cdeg, b.coarse_off,
                b.coarse_inv, b.coarse_ok);
        n += 1;
    }
    for (int l = L - 2; l >= 0; l--) {
        if (!any_level(l)) continue;
        const float *rin = (l == 0) ? b.r : b.mb;
        const int flo = b.lvl_prob_lo[l], fhi = b.lvl_prob_hi[l];
        int64_t maxnodes = 1;
        for (int pi = flo; pi < fhi; pi++)
            if (b.h_probs[pi].coarse >= 0)
                maxnodes = std::max<int64_t>(maxnodes, (int64_t)b.h_probs[pi].NX * b.h_probs[pi].NY * b.h_probs[pi].NZ);
        dim3 grid(std::max(1u, std::min(blocks_for(maxnodes, 256), 4096u)), fhi - flo);
        launch_pdl(mg_prolong_kernel, grid, 256, 0, b.stream, b.probs, flo, b.states, b.mx, b.dinv);
        launch_level_op<2>(b, fac, prec, l, 4, b.mx, rin, b.my, 0);  // my = rin - A mx
        n += 2 + enqueue_smooth(b, fac, prec, l, b.my, 0, sdeg, cs, 0);
    }
    return n;
}

// One solver step over every problem of the batch; each kernel acts only on the
// problems in its phase, so problems advance independently:
//   FP64 residual + stop test (RESID) | inner CG start (INIT) |
//   [multigrid z = M r, rz, beta] | p, q = A p, alpha | x, r, stop test |
//   u += d of stopped inner solves | phase transitions.
long long enqueue_step(MfBatch &b, const MfSolveParams &prm, int parity) {
    cudaStream_t s = b.stream;
    const int n0 = b.lvl_chunk_hi[0], nb0 = b.lvl_brick_hi[0];
    const int vg0 = std::max(1, std::min(n0, b.vec_grid));
    const bool use_mg = prm.mg && b.n_levels > 1;
    const int maxit = prm.max_iterations > 0 ? prm.max_iterations : 100000;
    const int max_ref = prm.max_refinements > 0 ? prm.max_refinements : 30;
    launch_pdl(mf_residual64_kernel, std::max(1, std::min(nb0, b.apply_grid)), kThreads, kResidSmem, s, 
        b.probs, b.bricks, nb0, b.Edf, b.node_fix, b.u64, b.f64, b.facdf, b.r64, b.states,
        b.brick_part, prm.rtol * prm.rtol, max_ref);
    launch_pdl(mf_inner_init_kernel, vg0, kThreads, 0, s, 
        b.chunks, n0, b.probs, b.r64, b.x, b.r, b.z, b.p0, b.p1, b.dinv, b.states, b.chunk_part,
        prm.inner_rtol * prm.inner_rtol, maxit);
    long long n = 2;
    float *pnew = parity ? b.p0 : b.p1;
    if (use_mg) {
        const int sdeg = prm.smooth_deg > 0 ? prm.smooth_deg : 2;
        const int cdeg = prm.coarse_deg > 0 ? prm.coarse_deg : 8;
        n += enqueue_vcycle(b, prm.mg_operator == 0, mg_precision(prm.precision), sdeg, cdeg);
        launch_pdl(mf_dot_rz_kernel, vg0, kThreads, 0, s, b.chunks, n0, b.probs, b.r, b.mx, b.states,
                                                 b.chunk_part, 0);
        launch_cg_apply(b, prm.precision, 4, parity);  // p = z + beta p_old, q = A p, alpha
        launch_update(b, pnew, true);                  // x, r, stop test
        n += 3;
    } else {
        launch_cg_apply(b, prm.precision, 0, parity);
        launch_update(b, pnew, false);                 // also z = D^-1 r, beta
        n += 2;
    }
    launch_pdl(mf_refine_kernel, vg0, kThreads, 0, s, b.chunks, n0, b.x, b.u64, b.states);
    launch_pdl(mf_phase_kernel, (b.n_fine + 127) / 128, 128, 0, s, b.states, b.n_fine);
    return n + 2;
}

// CUDA graph of `chunk` solver steps (even: the p0/p1 roles alternate per step),
// cached per parameter set
int build_step_graph(MfBatch &b, const MfSolveParams &prm, int chunk) {
    const std::vector<double> key = {(double)prm.precision, (double)chunk, (double)prm.mg,
                                     (double)prm.smooth_deg, (double)prm.coarse_deg, prm.rtol,
                                     prm.inner_rtol, (double)prm.max_iterations,
                                     (double)prm.max_refinements, (double)b.vec_grid,
                                     (double)prm.mg_operator};
    if (b.graph && b.graph_key == key) return MG_OK;
    if (b.graph) {
        cudaGraphExecDestroy(b.graph);
        b.graph = nullptr;
    }
    long long n = 0;
    cudaGraph_t g = nullptr;
    b.enqueue_error = 0;
    MG_CUDA_TRY(cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal));
    for (int it = 0; it < chunk; it++) n += enqueue_step(b, prm, it & 1);
    cudaError_t e = cudaStreamEndCapture(b.stream, &g);
    if (e != cudaSuccess) {
        set_error("graph capture: %s", cudaGetErrorString(e));
        return MG_ECUDA;
    }
    if (b.enqueue_error) {
        cudaGraphDestroy(g);
        set_error("factored level operator: a vector without a tensor map");
        return b.enqueue_error;
    }
    e = cudaGraphInstantiate(&b.graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b.graph = nullptr;
        set_error("graph instantiate: %s", cudaGetErrorString(e));
        return MG_ECUDA;
    }
    b.graph_key = key;
    b.graph_launches = n;
    return MG_OK;
}

}  // namespace

// FP64 iterative refinement around FP32 tensor-core CG, per problem:
//   r = f - K u (FP64);  stop when ||r|| <= rtol ||f||;
//   solve A d = r / ||r|| with FP32 CG to inner_rtol (Jacobi or multigrid
//   V-cycle preconditioned);  u += ||r|| d.
// The phases run on the device (enqueue_step); the host only relaunches the
// step graph until every active problem has finished.
int mf_batch_prepare(MfBatch &b, const MfSolveParams &prm) {
    const bool use_mg = prm.mg && b.n_levels > 1;
    // launch shape of the vector kernels (captured in the graph)
    int dev = 0, sms = 0;
    MG_CUDA_TRY(cudaGetDevice(&dev));
    MG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int per_sm = prm.vec_blocks_per_sm > 0 ? std::min(prm.vec_blocks_per_sm, 64) : 8;
    const int vg = std::max(1, std::min(b.n_chunks, per_sm * sms));
    if (vg != b.vec_grid) {
        b.vec_grid = vg;
        if (b.graph) cudaGraphExecDestroy(b.graph);
        b.graph = nullptr;
    }
    const int chunk = prm.graph_chunk > 0 ? (prm.graph_chunk + 1) / 2 * 2 : (use_mg ? 2 : 16);
    MfSolveParams p2 = prm;
    p2.mg = use_mg ? 1 : 0;
    return build_step_graph(b, p2, chunk);
}

int mf_batch_reset_states(MfBatch &b) {
    std::vector<MfState> init(b.n_probs);
    memset(init.data(), 0, init.size() * sizeof(MfState));
    for (int i = 0; i < b.n_probs; i++) {
        init[i].done = 1;
        init[i].ref_done = 1;
        init[i].phase = kPhaseFin;
    }
    MG_CUDA_TRY(cudaMemcpyAsync(b.states, init.data(), b.n_probs * sizeof(MfState), cudaMemcpyHostToDevice,
                                b.stream));
    MG_CUDA_TRY(cudaStreamSynchronize(b.stream));  // init is a host temporary
    memcpy(b.states_host, init.data(), b.n_probs * sizeof(MfState));
    return MG_OK;
}

int mf_batch_activate(MfBatch &b, const std::vector<int> &level0, bool warm_start) {
    MG_TRY(compute_diag_list(b, level0));
    for (int i : level0) {
        if (i < 0 || i >= b.n_fine) return MG_EINVAL;
        const MfProblem &P = b.h_probs[i];
        if (!warm_start) MG_CUDA_TRY(cudaMemsetAsync(b.u64 + P.dof_off, 0, P.n_pad * 8, b.stream));
        // the pinned host mirror entry is the staging buffer; the next
        // read_states (later in stream order) overwrites it
        MfState &h = b.states_host[i];
        memset(&h, 0, sizeof(MfState));
        h.done = 1;
        h.phase = kPhaseResid;  // its first residual pass also forms ||f||^2
        h.u_zero = warm_start ? 0 : 1;
        MG_CUDA_TRY(cudaMemcpyAsync(b.states + i, &h, sizeof(MfState), cudaMemcpyHostToDevice, b.stream));
    }
    return MG_OK;
}

int mf_batch_step(MfBatch &b) {
    if (!b.graph) {
        set_error("mf_batch_step before mf_batch_prepare");
        return MG_EINVAL;
    }
    MG_CUDA_TRY(cudaGraphLaunch(b.graph, b.stream));
    count_launches(b.graph_launches);
    return read_states(b);  // synchronises
}

int mf_batch_step_begin(MfBatch &b) {
    if (!b.graph) {
        set_error("mf_batch_step before mf_batch_prepare");
        return MG_EINVAL;
    }
    if (!b.err_host) MG_CUDA_TRY(cudaMallocHost(&b.err_host, sizeof(int)));
    MG_CUDA_TRY(cudaGraphLaunch(b.graph, b.stream));
    count_launches(b.graph_launches);
    MG_CUDA_TRY(cudaMemcpyAsync(b.states_host, b.states, b.n_probs * sizeof(MfState), cudaMemcpyDeviceToHost,
                                b.stream));
    MG_CUDA_TRY(cudaMemcpyAsync(b.err_host, b.err, sizeof(int), cudaMemcpyDeviceToHost, b.stream));
    return MG_OK;
}

int mf_batch_step_end(MfBatch &b) {
    MG_CUDA_TRY(cudaStreamSynchronize(b.stream));
    if (*b.err_host) {
        set_error("tensor-core pipeline wait exceeded its bound (error flag %d)", *b.err_host);
        return MG_ETIMEDOUT;
    }
    return MG_OK;
}

int mf_batch_finish(MfBatch &b, int i) {
    // a zero load gives u = 0 (the residual pass marks it with ||f||^2 = -1)
    if (b.states_host[i].ff64 < 0.0)
        MG_CUDA_TRY(cudaMemsetAsync(b.u64 + b.h_probs[i].dof_off, 0, b.h_probs[i].n_pad * 8, b.stream));
    return b.states_host[i].ref_status;
}

int mf_batch_solve(MfBatch &b, const MfSolveParams &prm, bool warm_start) {
    const double t0 = wall_time();
    MG_TRY(mf_batch_prepare(b, prm));
    MG_TRY(mf_batch_reset_states(b));
    std::vector<int> act;
    for (int i = 0; i < b.n_fine; i++)
        if (!prm.active || prm.active[i]) act.push_back(i);
    MG_TRY(mf_batch_activate(b, act, warm_start));
    for (;;) {
        MG_TRY(mf_batch_step(b));
        bool all_done = true;
        for (int i : act) all_done &= b.states_host[i].phase == kPhaseFin;
        if (all_done) break;
        if (prm.timeout_s > 0 && wall_time() - t0 > prm.timeout_s) {
            set_error("mixed solve exceeded %.1f s", prm.timeout_s);
            return MG_ETIMEDOUT;
        }
    }
    int rc = MG_OK;
    for (int i : act) {
        const int st = mf_batch_finish(b, i);
        if (st != 0 && rc == MG_OK) rc = st;
    }
    return rc;
}

// compliance f.u per design (host) and dC/drho (unpadded, designs back to back
// in problem order at dc_unpadded_dev) from the resident solutions
int mf_batch_compliance(MfBatch &b, double *compliance_host, double *dc_unpadded_dev,
                        const uint8_t *active) {
    cudaStream_t s = b.stream;
    const int n0 = b.lvl_chunk_hi[0];
    if (compliance_host) {
        mf_dot_chunks_kernel<<<std::max(1, std::min(n0, b.vec_grid)), kThreads, 0, s>>>(
            b.chunks, n0, b.f64, b.u64, b.chunk_part);
        MG_CUDA_TRY(cudaGetLastError());
        std::vector<double> part(n0);
        MG_CUDA_TRY(cudaMemcpyAsync(part.data(), b.chunk_part, n0 * 8, cudaMemcpyDeviceToHost, s));
        MG_CUDA_TRY(cudaStreamSynchronize(s));
        for (int i = 0; i < b.n_fine; i++) {
            const MfProblem &P = b.h_probs[i];
            double c = 0;
            for (int k = 0; k < P.chunk_count; k++) c += part[P.chunk_begin + k];
            compliance_host[i] = c;
        }
    }
    if (dc_unpadded_dev) {
        // output offsets through the batch's pinned staging (free again when this returns)
        int64_t *offs = b.sens_offs_host;
        int64_t o = 0, max_ne = 1;
        for (int i = 0; i < b.n_fine; i++) {
            const MfProblem &P = b.h_probs[i];
            offs[i] = (active && !active[i]) ? -1 : o;  // -1: leave this problem's output
            o += (int64_t)P.nx * P.ny * P.nz;
            max_ne = std::max<int64_t>(max_ne, (int64_t)P.nx * P.ny * P.nz);
        }
        MG_CUDA_TRY(cudaMemcpyAsync(b.sens_offs, offs, b.n_fine * 8, cudaMemcpyHostToDevice, s));
        dim3 grid(std::max(1u, std::min(blocks_for(max_ne, 128), 4096u)), b.n_fine);
        mf_sens_kernel<<<grid, 128, 0, s>>>(b.probs, b.n_fine, b.dE64, b.node_fix, b.u64, b.facdf,
                                            b.sens_offs, dc_unpadded_dev);
        cudaError_t e = cudaGetLastError();
        cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("sensitivity kernel: %s", cudaGetErrorString(e));
            return MG_ECUDA;
        }
    }
    return MG_OK;
}

// ----------------------------------------------------- single-problem mixed path
struct MatfreeWork {
    MfBatch batch;
};

namespace {

int matfree_setup(mg_problem *p) {
    if (p->mf) return MG_OK;
    if (p->physics != MG_PHYSICS_ELASTICITY_HEX8 || p->grid_nx <= 0 || p->grid_ny <= 0 ||
        p->grid_nz <= 0 || (int64_t)p->grid_nx * p->grid_ny * p->grid_nz != p->n_elems) {
        set_error("the mixed form needs the structured HEX8 grid (grid dims)");
        return MG_ENOTSUP;
    }
    const int nx = p->grid_nx, ny = p->grid_ny, nz = p->grid_nz;
    // the grid must be uniform: coords(i,j,k) = (i hx, j hy, k hz) + origin
    const double *c = p->h_coords.data();
    const int64_t NX = nx + 1, NY = ny + 1;
    const double hx = c[3] - c[0], hy = c[NX * 3 + 1] - c[1], hz = c[NX * NY * 3 + 2] - c[2];
    for (int64_t n = 0; n < p->n_nodes; n++) {
        const int64_t i = n % NX, j = (n / NX) % NY, k = n / (NX * NY);
        if (fabs(c[n * 3] - (c[0] + i * hx)) > 1e-9 * (1 + fabs(hx) * nx) ||
            fabs(c[n * 3 + 1] - (c[1] + j * hy)) > 1e-9 * (1 + fabs(hy) * ny) ||
            fabs(c[n * 3 + 2] - (c[2] + k * hz)) > 1e-9 * (1 + fabs(hz) * nz)) {
            set_error("mesh is not a uniform structured grid");
            return MG_ENOTSUP;
        }
    }
    for (int64_t e = 0; e < p->n_elems; e++) {
        const int64_t i = e % nx, j = (e / nx) % ny, k = e / ((int64_t)nx * ny);
        if (p->h_conn[e * 8] != (int32_t)(i + NX * (j + NY * k))) {
            set_error("connectivity is not the libMesh grid numbering");
            return MG_ENOTSUP;
        }
    }
    MatfreeWork *w = new MatfreeWork();
    MfProblem P{};
    P.nx = nx; P.ny = ny; P.nz = nz;
    P.share_elems = -1;
    int rc = mf_batch_init(w->batch, {P}, hx, hy, hz, p->mat.nu, p->stream, kMaxLevels, true);
    if (rc == MG_OK) {
        std::vector<uint8_t> nf(p->n_nodes, 0);
        for (int64_t n = 0; n < p->n_nodes; n++)
            for (int cc = 0; cc < 3; cc++)
                if (p->h_fixed[n * 3 + cc]) nf[n] |= (uint8_t)(1u << cc);
        rc = mf_batch_set_bc(w->batch, 0, nf.data(), p->h_F.data());
    }
    if (rc != MG_OK) {
        mf_batch_free(w->batch);
        delete w;
        return rc;
    }
    p->mf = w;
    return MG_OK;
}

}  // namespace

int matfree_solve(mg_problem *p, const mg_solve_opts &o, mg_solve_report *rep, bool x_zero) {
    MG_TRY(matfree_setup(p));
    MfBatch &b = p->mf->batch;
    MG_TRY(mf_batch_set_moduli(b, 0, p->d_E, p->d_dE));
    if (!x_zero) {
        MG_TRY(mf_batch_set_u(b, 0, p->d_X));
        count_launches(1);
    }
    MfSolveParams prm;
    prm.precision = o.precision;
    prm.rtol = o.rtol;
    prm.inner_rtol = o.inner_rtol > 0 ? o.inner_rtol : 1e-4;
    prm.max_iterations = o.max_iterations;
    prm.max_refinements = o.max_refinements;
    prm.graph_chunk = o.graph_chunk;
    prm.timeout_s = o.timeout_s;
    prm.mg = (o.preconditioner == MG_PC_MULTIGRID) ? 1 : 0;
    prm.smooth_deg = o.smooth_degree;
    prm.coarse_deg = o.coarse_degree;
    prm.vec_blocks_per_sm = o.vec_blocks_per_sm;
    prm.mg_operator = o.smoother_operator == MG_SMOOTHER_TENSOR ? 1 : 0;
    // from 0 (activation clears u): the first residual is f without an operator pass
    int rc = mf_batch_solve(b, prm, !x_zero);
    MG_TRY(mf_batch_get_u(b, 0, p->d_X));
    count_launches(1);
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    const MfState &h = b.states_host[0];
    if (rep) {
        rep->newton_iterations = 1;
        rep->krylov_iterations = h.total_iter;
        rep->refinements = h.refine;
        rep->relres = h.ff64 > 0.0 ? sqrt(h.rr64 / h.ff64) : 0.0;
        rep->residual_norm = sqrt(h.rr64);
    }
    return rc;
}

int matfree_apply_debug(mg_problem *p, int precision, const double *x_host, double *y_host) {
    MG_TRY(matfree_setup(p));
    MfBatch &b = p->mf->batch;
    MG_TRY(mf_batch_set_moduli(b, 0, p->d_E, p->d_dE));
    return mf_apply(b, precision, x_host, y_host, 0);
}

// dC/drho from the resident solution with the shared K0 (FP64)
int matfree_sensitivity(mg_problem *p, double *dc_host) {
    MG_TRY(matfree_setup(p));
    MfBatch &b = p->mf->batch;
    MG_TRY(mf_batch_set_moduli(b, 0, p->d_E, p->d_dE));
    MG_TRY(mf_batch_set_u(b, 0, p->d_X));
    MG_TRY(mf_batch_compliance(b, nullptr, p->d_elem_out));
    MG_CUDA_TRY(cudaMemcpyAsync(dc_host, p->d_elem_out, p->n_elems * 8, cudaMemcpyDeviceToHost, p->stream));
    MG_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return MG_OK;
}

int matfree_compliance_resident(mg_problem *p, double *compliance) {
    MG_TRY(matfree_setup(p));
    MfBatch &b = p->mf->batch;
    double c = 0.0;
    MG_TRY(mf_batch_compliance(b, &c, p->d_elem_out));
    count_launches(2);
    if (compliance) *compliance = c;
    return MG_OK;
}

int matfree_launch_apply(mg_problem *p, int precision, int reps) {
    MG_TRY(matfree_setup(p));
    MfBatch &b = p->mf->batch;
    MG_TRY(mf_batch_set_moduli(b, 0, p->d_E, p->d_dE));
    return mf_launch_apply(b, precision, reps);
}

void matfree_free(mg_problem *p) {
    if (!p->mf) return;
    mf_batch_free(p->mf->batch);
    delete p->mf;
    p->mf = nullptr;
}

}  // namespace mg
