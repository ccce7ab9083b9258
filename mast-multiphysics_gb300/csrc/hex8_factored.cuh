// Factored HEX8 box-element stiffness for the CUDA-core operators.
//
// On a box element (edges hx, hy, hz; isotropic material) the trilinear shape
// functions are products of 1D hats, and every 1D factor of the stiffness
// integrals (mass, stiffness and mixed derivative matrices of a 2-node line) is
// diagonal or anti-diagonal in the per-axis sum/difference basis
// (s = u1 + u0, d = u1 - u0).  In that basis K0 has 45 nonzeros of 576
// (rigid translations, mode 0, are in the kernel), so
//     K0 u_e = P^T H (Khat / 64) H^T P u_e
// with H^T the 3-stage butterfly (8-point Walsh-Hadamard transform) of each
// displacement component and P the corner permutation from the element's node
// order (StructuralElement3D / libMesh HEX8: corner a = (dx, dy, dz) with
// a = 0..3 counter-clockwise at z = 0, 4..7 at z = 1) to the lexicographic
// corner index b = bx + 2 by + 4 bz.  One element costs 2 x 72 butterfly
// additions and 45 FMA instead of the 576 FMA of the dense 24 x 24 product.
// Khat is formed on the host from the same K0 the other kernels use
// (hex8_factored_build), which also checks that the 531 other entries vanish.
#pragma once

#include <cstdint>

namespace mg {

constexpr int kFacN = 45;

template <typename T>
struct FacK {
    T v[kFacN];  // entry k of Khat / 64, in the order of kFacTerms
};

// (out component, out mode, in component, in mode) of each nonzero of Khat
static const int kFacTerms[kFacN][4] = {
    {0, 1, 0, 1}, {0, 1, 1, 2}, {0, 1, 2, 4}, {0, 2, 0, 2}, {0, 2, 1, 1}, {0, 3, 0, 3}, {0, 3, 2, 6},
    {0, 4, 0, 4}, {0, 4, 2, 1}, {0, 5, 0, 5}, {0, 5, 1, 6}, {0, 6, 0, 6}, {0, 6, 1, 5}, {0, 6, 2, 3},
    {0, 7, 0, 7}, {1, 1, 0, 2}, {1, 1, 1, 1}, {1, 2, 0, 1}, {1, 2, 1, 2}, {1, 2, 2, 4}, {1, 3, 1, 3},
    {1, 3, 2, 5}, {1, 4, 1, 4}, {1, 4, 2, 2}, {1, 5, 0, 6}, {1, 5, 1, 5}, {1, 5, 2, 3}, {1, 6, 0, 5},
    {1, 6, 1, 6}, {1, 7, 1, 7}, {2, 1, 0, 4}, {2, 1, 2, 1}, {2, 2, 1, 4}, {2, 2, 2, 2}, {2, 3, 0, 6},
    {2, 3, 1, 5}, {2, 3, 2, 3}, {2, 4, 0, 1}, {2, 4, 1, 2}, {2, 4, 2, 4}, {2, 5, 1, 3}, {2, 5, 2, 5},
    {2, 6, 0, 3}, {2, 6, 2, 6}, {2, 7, 2, 7}};

// Khat / 64 from a node-interleaved K0 (dof 3a + c, a in element node order);
// returns false if an entry outside the 45-term pattern is not negligible
// (K0 is then not a box-element stiffness of an isotropic material)
inline bool hex8_factored_build(const double *K0, FacK<double> &k64, FacK<float> &k32) {
    auto corner_of_lex = [](int b) {  // lexicographic corner -> element node order
        const int bx = b & 1, by = (b >> 1) & 1, bz = (b >> 2) & 1;
        return bz * 4 + (by ? (bx ? 2 : 3) : (bx ? 1 : 0));
    };
    auto sgn = [](int m, int b) {  // H[b][m]: +1 / -1
        int s = 1;
        for (int t = 0; t < 3; t++)
            if ((m >> t) & 1) s *= ((b >> t) & 1) ? 1 : -1;
        return s;
    };
    double kh[3][8][3][8];
    double vmax = 0.0;
    for (int c = 0; c < 3; c++)
        for (int m = 0; m < 8; m++)
            for (int d = 0; d < 3; d++)
                for (int mm = 0; mm < 8; mm++) {
                    double s = 0.0;
                    for (int b = 0; b < 8; b++)
                        for (int bb = 0; bb < 8; bb++)
                            s += sgn(m, b) * sgn(mm, bb) *
                                 K0[(3 * corner_of_lex(b) + c) * 24 + 3 * corner_of_lex(bb) + d];
                    kh[c][m][d][mm] = s / 64.0;
                    vmax = s / 64.0 > vmax ? s / 64.0 : (-s / 64.0 > vmax ? -s / 64.0 : vmax);
                }
    bool in_pattern[3][8][3][8] = {};
    for (int k = 0; k < kFacN; k++) {
        const int *t = kFacTerms[k];
        in_pattern[t[0]][t[1]][t[2]][t[3]] = true;
        k64.v[k] = kh[t[0]][t[1]][t[2]][t[3]];
        k32.v[k] = (float)k64.v[k];
    }
    for (int c = 0; c < 3; c++)
        for (int m = 0; m < 8; m++)
            for (int d = 0; d < 3; d++)
                for (int mm = 0; mm < 8; mm++) {
                    const double a = kh[c][m][d][mm];
                    if (!in_pattern[c][m][d][mm] && (a > 1e-12 * vmax || -a > 1e-12 * vmax)) return false;
                }
    return true;
}

// Double-float number: the unevaluated sum hi + lo of two FP32 values with
// |lo| <= ulp(hi) / 2, a 48-bit significand carried on the FP32 pipes (GB300's
// FP64 pipe issues two DFMA per cycle per SM, its FP32 pipes 128 FFMA).  The
// operations are the classical error-free transformations: Knuth's two-sum for
// additions and the FMA form of Dekker's two-product for products, each followed
// by a renormalising fast two-sum.  Explicitly rounded intrinsics keep the
// compiler from contracting or reassociating them.
struct dfloat {
    float hi, lo;
};

inline dfloat dfloat_of(double x) {
    dfloat r;
    r.hi = (float)x;
    r.lo = (float)(x - (double)r.hi);
    return r;
}

#ifdef __CUDACC__
__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }

__device__ __forceinline__ dfloat df_renorm(float s, float e) {
    dfloat r;
    r.hi = __fadd_rn(s, e);
    r.lo = __fsub_rn(e, __fsub_rn(r.hi, s));
    return r;
}
__device__ __forceinline__ dfloat operator+(dfloat a, dfloat b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    return df_renorm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dfloat operator-(dfloat a, dfloat b) {
    dfloat nb;
    nb.hi = -b.hi;
    nb.lo = -b.lo;
    return a + nb;
}
__device__ __forceinline__ dfloat operator*(dfloat a, dfloat b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return df_renorm(p, e);
}
__device__ __forceinline__ dfloat &operator+=(dfloat &a, dfloat b) { return a = a + b; }
__device__ __forceinline__ dfloat &operator*=(dfloat &a, dfloat b) { return a = a * b; }
__device__ __forceinline__ dfloat fma_t(dfloat a, dfloat b, dfloat c) { return a * b + c; }
__device__ __forceinline__ dfloat df_from(double x) {
    dfloat r;
    r.hi = __double2float_rn(x);
    r.lo = __double2float_rn(x - (double)r.hi);
    return r;
}
__device__ __forceinline__ double df_to(dfloat a) { return (double)a.hi + (double)a.lo; }
// df_from by integer operations on the bits of x (the FP64 pipe stays free):
// hi = x rounded to nearest even at 24 bits, lo = x - hi (exact) rounded to
// nearest, the same pair as df_from.  Zeros give (0, 0); magnitudes outside
// [2^-74, 2^100) (where lo would not be a normal float) take df_from.
__device__ __forceinline__ dfloat df_split(double x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    dfloat r;
    if ((b << 1) == 0ull) {
        r.hi = 0.0f;
        r.lo = 0.0f;
        return r;
    }
    const int e = (int)((b >> 52) & 0x7FFull);
    if (e < 949 || e > 1122) return df_from(x);
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);  // x = m 2^(e - 1075)
    unsigned long long q = m >> 29;
    const unsigned long long rem = m & ((1ull << 29) - 1ull);
    if (rem > (1ull << 28) || (rem == (1ull << 28) && (q & 1ull))) q++;
    const int d = (int)((long long)m - (long long)(q << 29));  // (x - hi) / 2^(e - 1075), |d| <= 2^28
    unsigned eh = (unsigned)(e - 1023 + 127), qh = (unsigned)q;
    if (qh == (1u << 24)) {
        qh >>= 1;
        eh += 1;
    }
    const unsigned sign = (unsigned)(b >> 63) << 31;
    r.hi = __uint_as_float(sign | (eh << 23) | (qh & 0x7FFFFFu));
    // 2^(e - 1075) is a normal float for e >= 949; d to float rounds once, the scaling is exact
    r.lo = __fmul_rn(__int2float_rn(sign ? -d : d), __uint_as_float((unsigned)(e - 1075 + 127) << 23));
    return r;
}
__device__ __forceinline__ dfloat df_zero() {
    dfloat r;
    r.hi = 0.0f;
    r.lo = 0.0f;
    return r;
}
template <typename T>
__device__ __forceinline__ T zero_t() { return T(0); }
template <>
__device__ __forceinline__ dfloat zero_t<dfloat>() { return df_zero(); }

// v[c][b]: component c at lexicographic corner b; on return its sum/difference
// modes u~ = H^T u (per component, the 8-point Walsh-Hadamard butterfly)
template <typename T>
__device__ __forceinline__ void hex8_factored_forward(T (&v)[3][8]) {
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int t = 1; t < 8; t <<= 1)
#pragma unroll
            for (int b = 0; b < 8; b++)
                if (!(b & t)) {
                    const T lo = v[c][b], hi = v[c][b | t];
                    v[c][b] = lo + hi;
                    v[c][b | t] = hi - lo;
                }
}

// yh[c][m] = (Khat / 64 u~)[c][m] for the modes m = 1..7 (mode 0, the rigid
// translation, is in the kernel: yh[c][0] is not set).  u_e^T K0 u_e equals the
// sum over c, m of u~[c][m] yh[c][m].
template <typename T>
__device__ __forceinline__ void hex8_factored_khat(const FacK<T> &K, const T (&v)[3][8], T (&yh)[3][8]) {
    yh[0][1] = K.v[0] * v[0][1];
    yh[0][1] = fma_t(K.v[1], v[1][2], yh[0][1]);
    yh[0][1] = fma_t(K.v[2], v[2][4], yh[0][1]);
    yh[0][2] = K.v[3] * v[0][2];
    yh[0][2] = fma_t(K.v[4], v[1][1], yh[0][2]);
    yh[0][3] = K.v[5] * v[0][3];
    yh[0][3] = fma_t(K.v[6], v[2][6], yh[0][3]);
    yh[0][4] = K.v[7] * v[0][4];
    yh[0][4] = fma_t(K.v[8], v[2][1], yh[0][4]);
    yh[0][5] = K.v[9] * v[0][5];
    yh[0][5] = fma_t(K.v[10], v[1][6], yh[0][5]);
    yh[0][6] = K.v[11] * v[0][6];
    yh[0][6] = fma_t(K.v[12], v[1][5], yh[0][6]);
    yh[0][6] = fma_t(K.v[13], v[2][3], yh[0][6]);
    yh[0][7] = K.v[14] * v[0][7];
    yh[1][1] = K.v[15] * v[0][2];
    yh[1][1] = fma_t(K.v[16], v[1][1], yh[1][1]);
    yh[1][2] = K.v[17] * v[0][1];
    yh[1][2] = fma_t(K.v[18], v[1][2], yh[1][2]);
    yh[1][2] = fma_t(K.v[19], v[2][4], yh[1][2]);
    yh[1][3] = K.v[20] * v[1][3];
    yh[1][3] = fma_t(K.v[21], v[2][5], yh[1][3]);
    yh[1][4] = K.v[22] * v[1][4];
    yh[1][4] = fma_t(K.v[23], v[2][2], yh[1][4]);
    yh[1][5] = K.v[24] * v[0][6];
    yh[1][5] = fma_t(K.v[25], v[1][5], yh[1][5]);
    yh[1][5] = fma_t(K.v[26], v[2][3], yh[1][5]);
    yh[1][6] = K.v[27] * v[0][5];
    yh[1][6] = fma_t(K.v[28], v[1][6], yh[1][6]);
    yh[1][7] = K.v[29] * v[1][7];
    yh[2][1] = K.v[30] * v[0][4];
    yh[2][1] = fma_t(K.v[31], v[2][1], yh[2][1]);
    yh[2][2] = K.v[32] * v[1][4];
    yh[2][2] = fma_t(K.v[33], v[2][2], yh[2][2]);
    yh[2][3] = K.v[34] * v[0][6];
    yh[2][3] = fma_t(K.v[35], v[1][5], yh[2][3]);
    yh[2][3] = fma_t(K.v[36], v[2][3], yh[2][3]);
    yh[2][4] = K.v[37] * v[0][1];
    yh[2][4] = fma_t(K.v[38], v[1][2], yh[2][4]);
    yh[2][4] = fma_t(K.v[39], v[2][4], yh[2][4]);
    yh[2][5] = K.v[40] * v[1][3];
    yh[2][5] = fma_t(K.v[41], v[2][5], yh[2][5]);
    yh[2][6] = K.v[42] * v[0][3];
    yh[2][6] = fma_t(K.v[43], v[2][6], yh[2][6]);
    yh[2][7] = K.v[44] * v[2][7];
}

// v[c][b]: component c at lexicographic corner b; on return e * (K0 u_e) in the
// same layout.  Fixed operation order (deterministic).
template <typename T>
__device__ __forceinline__ void hex8_factored_apply(const FacK<T> &K, T e, T (&v)[3][8]) {
    hex8_factored_forward(v);
    T yh[3][8];
    hex8_factored_khat(K, v, yh);
    // back to the corners: the transpose butterflies, mode 0 is zero
#pragma unroll
    for (int c = 0; c < 3; c++) {
        yh[c][0] = zero_t<T>();
#pragma unroll
        for (int m = 1; m < 8; m++) yh[c][m] *= e;
#pragma unroll
        for (int t = 1; t < 8; t <<= 1)
#pragma unroll
            for (int b = 0; b < 8; b++)
                if (!(b & t)) {
                    const T a = yh[c][b], bb = yh[c][b | t];
                    yh[c][b] = a - bb;
                    yh[c][b | t] = a + bb;
                }
#pragma unroll
        for (int b = 0; b < 8; b++) v[c][b] = yh[c][b];
    }
}

// Two elements at once in packed FP32x2 arithmetic (each component of a
// float2 is one element; per component the same operations, in the same
// order and rounding, as hex8_factored_apply<float>)
struct FacK2 {
    float2 v[kFacN];  // (k, k) pairs of FacK<float>
};

__device__ __forceinline__ void hex8_factored_apply2(const FacK2 &K, float2 e, float2 (&v)[3][8]) {
    const float2 m1 = make_float2(-1.0f, -1.0f);
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int t = 1; t < 8; t <<= 1)
#pragma unroll
            for (int b = 0; b < 8; b++)
                if (!(b & t)) {
                    const float2 lo = v[c][b], hi = v[c][b | t];
                    v[c][b] = __fadd2_rn(lo, hi);
                    v[c][b | t] = __ffma2_rn(lo, m1, hi);  // hi - lo
                }
    float2 yh[3][8];
    yh[0][1] = __fmul2_rn(K.v[0], v[0][1]);
    yh[0][1] = __ffma2_rn(K.v[1], v[1][2], yh[0][1]);
    yh[0][1] = __ffma2_rn(K.v[2], v[2][4], yh[0][1]);
    yh[0][2] = __fmul2_rn(K.v[3], v[0][2]);
    yh[0][2] = __ffma2_rn(K.v[4], v[1][1], yh[0][2]);
    yh[0][3] = __fmul2_rn(K.v[5], v[0][3]);
    yh[0][3] = __ffma2_rn(K.v[6], v[2][6], yh[0][3]);
    yh[0][4] = __fmul2_rn(K.v[7], v[0][4]);
    yh[0][4] = __ffma2_rn(K.v[8], v[2][1], yh[0][4]);
    yh[0][5] = __fmul2_rn(K.v[9], v[0][5]);
    yh[0][5] = __ffma2_rn(K.v[10], v[1][6], yh[0][5]);
    yh[0][6] = __fmul2_rn(K.v[11], v[0][6]);
    yh[0][6] = __ffma2_rn(K.v[12], v[1][5], yh[0][6]);
    yh[0][6] = __ffma2_rn(K.v[13], v[2][3], yh[0][6]);
    yh[0][7] = __fmul2_rn(K.v[14], v[0][7]);
    yh[1][1] = __fmul2_rn(K.v[15], v[0][2]);
    yh[1][1] = __ffma2_rn(K.v[16], v[1][1], yh[1][1]);
    yh[1][2] = __fmul2_rn(K.v[17], v[0][1]);
    yh[1][2] = __ffma2_rn(K.v[18], v[1][2], yh[1][2]);
    yh[1][2] = __ffma2_rn(K.v[19], v[2][4], yh[1][2]);
    yh[1][3] = __fmul2_rn(K.v[20], v[1][3]);
    yh[1][3] = __ffma2_rn(K.v[21], v[2][5], yh[1][3]);
    yh[1][4] = __fmul2_rn(K.v[22], v[1][4]);
    yh[1][4] = __ffma2_rn(K.v[23], v[2][2], yh[1][4]);
    yh[1][5] = __fmul2_rn(K.v[24], v[0][6]);
    yh[1][5] = __ffma2_rn(K.v[25], v[1][5], yh[1][5]);
    yh[1][5] = __ffma2_rn(K.v[26], v[2][3], yh[1][5]);
    yh[1][6] = __fmul2_rn(K.v[27], v[0][5]);
    yh[1][6] = __ffma2_rn(K.v[28], v[1][6], yh[1][6]);
    yh[1][7] = __fmul2_rn(K.v[29], v[1][7]);
    yh[2][1] = __fmul2_rn(K.v[30], v[0][4]);
    yh[2][1] = __ffma2_rn(K.v[31], v[2][1], yh[2][1]);
    yh[2][2] = __fmul2_rn(K.v[32], v[1][4]);
    yh[2][2] = __ffma2_rn(K.v[33], v[2][2], yh[2][2]);
    yh[2][3] = __fmul2_rn(K.v[34], v[0][6]);
    yh[2][3] = __ffma2_rn(K.v[35], v[1][5], yh[2][3]);
    yh[2][3] = __ffma2_rn(K.v[36], v[2][3], yh[2][3]);
    yh[2][4] = __fmul2_rn(K.v[37], v[0][1]);
    yh[2][4] = __ffma2_rn(K.v[38], v[1][2], yh[2][4]);
    yh[2][4] = __ffma2_rn(K.v[39], v[2][4], yh[2][4]);
    yh[2][5] = __fmul2_rn(K.v[40], v[1][3]);
    yh[2][5] = __ffma2_rn(K.v[41], v[2][5], yh[2][5]);
    yh[2][6] = __fmul2_rn(K.v[42], v[0][3]);
    yh[2][6] = __ffma2_rn(K.v[43], v[2][6], yh[2][6]);
    yh[2][7] = __fmul2_rn(K.v[44], v[2][7]);
#pragma unroll
    for (int c = 0; c < 3; c++) {
#pragma unroll
        for (int m = 1; m < 8; m++) yh[c][m] = __fmul2_rn(yh[c][m], e);
        yh[c][0] = make_float2(0.0f, 0.0f);  // mode 0 is zero
#pragma unroll
        for (int t = 1; t < 8; t <<= 1)
#pragma unroll
            for (int b = 0; b < 8; b++)
                if (!(b & t)) {
                    const float2 a = yh[c][b], bb = yh[c][b | t];
                    yh[c][b] = __ffma2_rn(bb, m1, a);  // a - bb
                    yh[c][b | t] = __fadd2_rn(a, bb);
                }
#pragma unroll
        for (int b = 0; b < 8; b++) v[c][b] = yh[c][b];
    }
}
#endif

}  // namespace mg
