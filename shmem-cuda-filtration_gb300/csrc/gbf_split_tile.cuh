// gbf_split_tile.cuh — the split-precision z-marching tile (device code);
// included by gbf_split.cu and gbf_ensemble.cu.
#pragma once

#include <math.h>

#include <type_traits>

#include "gbf_split.h"
#include "gbf_tma.h"

// ------------------------------------------------------------ FP32 pairs
// Unevaluated sums hi + lo of two FP32 numbers ("double-float", about 48
// significant bits) built on the error-free transformations TwoSum (Knuth,
// TAOCP vol. 2, sec. 4.2.2), FastTwoSum (Dekker 1971) and TwoProduct through
// FMA. Used for the phase masses and the residual in GBF_PREC_SPLIT_DF.
struct GbfDF {
  float hi, lo;
};
__device__ __forceinline__ GbfDF df_two_sum(float a, float b) {
  float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ GbfDF df_fast_two_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ GbfDF df_add(GbfDF a, GbfDF b) {
  GbfDF s = df_two_sum(a.hi, b.hi);
  return df_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ GbfDF df_neg(GbfDF a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ GbfDF df_mul(GbfDF a, GbfDF b) {
  float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return df_fast_two_sum(p, e);
}
// a / b for an FP32 divisor: one correction of the FP32 quotient.
__device__ __forceinline__ GbfDF df_div_f(GbfDF a, float b) {
  const float q1 = __fdiv_rn(a.hi, b);
  const float p = __fmul_rn(q1, b), pe = __fmaf_rn(q1, b, -p);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), a.lo);
  return df_fast_two_sum(q1, __fdiv_rn(r, b));
}
__host__ __device__ __forceinline__ float2 gbf_df_from_double(double d) {
  float h = (float)d;
  return make_float2(h, (float)(d - (double)h));
}

// Wide arithmetic of the masses and the residual: FP64 or FP32 pairs.
template <bool DF> struct Wide;
template <> struct Wide<false> {
  using T = double;
  static __device__ __forceinline__ T f(float x) { return (double)x; }
  static __device__ __forceinline__ T c(double d, float2) { return d; }
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  static __device__ __forceinline__ T div_f(T a, float b) { return a / (double)b; }
  static __device__ __forceinline__ T mulf(T a, float b) { return a * (double)b; }
  static __device__ __forceinline__ float tof(T a) { return (float)a; }
  static __device__ __forceinline__ double tod(T a) { return a; }
  static __device__ __forceinline__ T load(const double* p, size_t i) { return p[i]; }
  static __device__ __forceinline__ void store(double* p, size_t i, T v) { p[i] = v; }
  // fused forms used by the tile (see the FP32-pair versions)
  static __device__ __forceinline__ T add_f(T a, float b) { return a + (double)b; }
  static __device__ __forceinline__ float rho_1mS_minus(T rho, T M, float S) {
    return (float)((rho - M) - rho * (double)S);
  }
  static __device__ __forceinline__ float rhoS_minus(T rho, T M, float S) { return (float)(rho * (double)S - M); }
  static __device__ __forceinline__ T acc_phi(T acc, float phi, T v) { return acc + (double)phi * v; }
};
template <> struct Wide<true> {
  using T = GbfDF;
  static __device__ __forceinline__ T f(float x) { return {x, 0.f}; }
  static __device__ __forceinline__ T c(double, float2 v) { return {v.x, v.y}; }
  static __device__ __forceinline__ T add(T a, T b) { return df_add(a, b); }
  static __device__ __forceinline__ T sub(T a, T b) { return df_add(a, df_neg(b)); }
  static __device__ __forceinline__ T mul(T a, T b) { return df_mul(a, b); }
  static __device__ __forceinline__ T div_f(T a, float b) { return df_div_f(a, b); }
  static __device__ __forceinline__ T mulf(T a, float b) {  // pair times FP32
    float p = a.hi * b;
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return df_fast_two_sum(p, e);
  }
  static __device__ __forceinline__ float tof(T a) { return a.hi + a.lo; }
  static __device__ __forceinline__ double tod(T a) { return (double)a.hi + (double)a.lo; }
  static __device__ __forceinline__ T load(const double* p, size_t i) {
    float2 v = reinterpret_cast<const float2*>(p)[i];
    return {v.x, v.y};
  }
  static __device__ __forceinline__ void store(double* p, size_t i, T v) {
    reinterpret_cast<float2*>(p)[i] = make_float2(v.hi, v.lo);
  }
  // pair + FP32: one TwoSum on the high parts, the rest folded into lo
  static __device__ __forceinline__ T add_f(T a, float b) {
    GbfDF s = df_two_sum(a.hi, b);
    return df_fast_two_sum(s.hi, s.lo + a.lo);
  }
  // (rho - M) - rho S rounded to FP32, with rho S exact (TwoProduct of the
  // high part plus the low part's product) and the large terms cancelled
  // by TwoSum before any rounding: rho (1 - S) - M of cpu.cpp:305.
  static __device__ __forceinline__ float rho_1mS_minus(T rho, T M, float S) {
    const GbfDF a = df_two_sum(rho.hi, -M.hi);                 // rho - M (high parts, exact)
    const float p = __fmul_rn(rho.hi, S), pe = __fmaf_rn(rho.hi, S, -p);  // rho.hi S, exact
    const GbfDF b = df_two_sum(a.hi, -p);
    return __fadd_rn(b.hi, __fadd_rn(b.lo, __fmaf_rn(-rho.lo, S, __fadd_rn(__fsub_rn(a.lo, pe),
                                                                            __fsub_rn(rho.lo, M.lo)))));
  }
  // rho S - M rounded to FP32 (cpu.cpp:306 without the small beta terms).
  static __device__ __forceinline__ float rhoS_minus(T rho, T M, float S) {
    const float p = __fmul_rn(rho.hi, S), pe = __fmaf_rn(rho.hi, S, -p);
    const GbfDF b = df_two_sum(p, -M.hi);
    return __fadd_rn(b.hi, __fadd_rn(b.lo, __fmaf_rn(rho.lo, S, __fsub_rn(pe, M.lo))));
  }
  // acc + phi v, the product's rounding error kept
  static __device__ __forceinline__ T acc_phi(T acc, float phi, T v) {
    const float p = v.hi * phi, pe = fmaf(v.hi, phi, -p);
    const GbfDF s = df_two_sum(acc.hi, p);
    return {s.hi, acc.lo + (s.lo + fmaf(v.lo, phi, pe))};
  }
};

// ------------------------------------------------- per-cell mass storage
// M1, M2 of the split forms: the phase masses in the wide type (kMassF64,
// kMassDF: 8 bytes a cell), or defects (below) in FP32 (kMassDefect, 4
// bytes) or FP32 pairs (kMassDefectDF, 8 bytes). The wide type of a form
// (constants, the source) is FP64 for kMassF64 and FP32 pairs otherwise.
template <int MR>
using WideOf = Wide<MR != kMassF64>;
template <int MR>
struct MassRep {
  using T = typename WideOf<MR>::T;
  static __device__ __forceinline__ T load(const double* p, size_t i) { return WideOf<MR>::load(p, i); }
  static __device__ __forceinline__ void store(double* p, size_t i, T v) { WideOf<MR>::store(p, i, v); }
};
template <>
struct MassRep<kMassDefect> {
  using T = float;
  static __device__ __forceinline__ T load(const double* p, size_t i) { return reinterpret_cast<const float*>(p)[i]; }
  static __device__ __forceinline__ void store(double* p, size_t i, T v) { reinterpret_cast<float*>(p)[i] = v; }
};
template <>
struct MassRep<kMassDefectDF> {
  using T = GbfDF;
  static __device__ __forceinline__ T load(const double* p, size_t i) { return Wide<true>::load(p, i); }
  static __device__ __forceinline__ void store(double* p, size_t i, T v) { Wide<true>::store(p, i, v); }
};
// A defect's FP32 value (the high part of a pair: |lo| <= ulp(hi) / 2) and
// a defect plus an FP32 increment, in each defect storage.
__device__ __forceinline__ float defect_f(float d) { return d; }
__device__ __forceinline__ float defect_f(GbfDF d) { return d.hi; }
__device__ __forceinline__ float defect_add(float d, float x) { return d + x; }
__device__ __forceinline__ GbfDF defect_add(GbfDF d, float x) { return Wide<true>::add_f(d, x); }
// Element type of a mass array in shared memory.
template <int MR>
using MassElem = typename std::conditional<MR == kMassDefect, float, double>::type;

// The defect form. A cell's phase masses per pore volume are held as
//   M1 = c1(j) (1 - S) + D1,   M2 = c2(j) S + D2,
// with S the cell's FP32 saturation, c_a(j) the hydrostatic density of phase
// a at row j, rho0a (1 + beta_a j H), rounded to FP32 (so c (1 - S) and c S
// are exact products), and D1, D2 "defects" (FP32, or FP32 pairs): the
// compressibility part rho0a beta_a dP and the Newton residual, small
// numbers. The residual of the Newton and the mass update then need FP32
// only, with rounding errors relative to those small numbers; e_a is the
// remainder rho0a (1 + beta_a j H) - c_a (FP32). Both follow from FP64 by
// fixed roundings, so every kernel derives the same values. Pair defects
// round at about 2^-48 |D| per update: with |D| / M <= 1e-2, finer than an
// FP64 mass's own rounding (2^-53 M).
struct GbfDefectRow {
  float c1, e1, c2, e2;
};
__device__ __forceinline__ GbfDefectRow gbf_defect_row(double ro01, double ro01b1, double ro02, double ro02b2,
                                                      double H, int j) {
  const double hs = __dmul_rn((double)j, H);
  const double r1 = __fma_rn(ro01b1, hs, ro01), r2 = __fma_rn(ro02b2, hs, ro02);
  GbfDefectRow w;
  w.c1 = __double2float_rn(r1);
  w.e1 = __double2float_rn(__dsub_rn(r1, (double)w.c1));
  w.c2 = __double2float_rn(r2);
  w.e2 = __double2float_rn(__dsub_rn(r2, (double)w.c2));
  return w;
}
// The same from the model (host-side gbf_split_consts forms ro0 beta and H
// with the same products).
__device__ __forceinline__ GbfDefectRow gbf_defect_row(const gbf_model& m, int j) {
  return gbf_defect_row(m.ro01, __dmul_rn(m.ro01, m.beta1), m.ro02, __dmul_rn(m.ro02, m.beta2),
                        __dmul_rn(__dmul_rn(m.ro01, m.g), m.h2), j);
}
__device__ __forceinline__ GbfDefectRow gbf_defect_row(const GbfSplitConsts& C, int j) {
  return gbf_defect_row(C.ro01_d, C.ro01b1_d, C.ro02_d, C.ro02b2_d, C.H_d, j);
}

// ------------------------------------------------------------- tile shape
// A CTA of TX x TY threads owns a TX x TY column tile (one column per thread).
// The halo plane (TX + 2 columns, TY + 2 rows) is stored with a row pitch PX
// >= TX + 2: TX + 2 for the plain-load tile, the TMA box width for the TMA
// tile (so that a halo element has the same index in the staged box).
template <int TX, int TY, int PX = TX + 2>
struct GbfSplitShape {
  static constexpr int threads = TX * TY;
  static constexpr int HX = PX, HY = TY + 2, HN = HX * HY;  // pitch, rows, elements
  static constexpr int slots = (HN + threads - 1) / threads;  // halo elements per thread
};
template <int TX, bool TMA>
__host__ __device__ constexpr int gbf_plane_pitch() { return TMA ? gbf_tma_box_x(TX) : TX + 2; }
// Default shape of the single-domain kernel.
constexpr int kSplitTX = 32, kSplitTY = 8;
constexpr int kSplitThreads = kSplitTX * kSplitTY;

// One x-y plane of the tile with its 1-cell halo.
template <int TX, int TY, int PX = TX + 2>
struct GbfSplitPlaneT {
  static constexpr int HN = GbfSplitShape<TX, TY, PX>::HN;
  float dP[HN], S[HN], L1[HN], L2[HN];
};
using GbfSplitPlane = GbfSplitPlaneT<kSplitTX, kSplitTY>;

// ----------------------------------------------------- TMA plane staging
// Two rings filled by cp.async.bulk.tensor, one mbarrier per stage:
//  - halo planes: dP, S, K of one x-y plane of the tile with its 1-cell halo,
//    up to kTmaStages planes ahead of the plane being built;
//  - interior rows: M1, M2 (8 bytes a cell, or 4 in the defect form) and
//    phi of the plane being updated, RS - 1 planes ahead (RS = 3 where the
//    static shared memory of the kernel stays within 48 KB, else 2).
// Every array starts on a 128-byte boundary.
constexpr int kTmaStages = 3;
template <int TX, int TY, int MR = kMassF64>
struct GbfRawRing {
  static constexpr int RS = TX >= 64 ? 2 : 3;
  static constexpr int BX = gbf_tma_box_x(TX), HY = TY + 2, N = BX * HY;
  static constexpr int NP = (N + 31) / 32 * 32;
  static constexpr int FX = gbf_tma_box_x(TX), NF = (FX * TY + 31) / 32 * 32;  // FP32 elements
  // mass rows: 8-byte elements {TX + 2, TY}, or FP32 ones in phi's box
  static constexpr int MB = (int)sizeof(MassElem<MR>);
  static constexpr int MX = MB == 8 ? gbf_tma_rows_x8(TX) : FX;
  static constexpr int NM = MB == 8 ? (MX * TY + 15) / 16 * 16 : NF;
  // bytes that complete one stage of each ring (whole boxes, also where they overhang the grid)
  static constexpr unsigned kHaloBytes = 3u * N * 4u;
  static constexpr unsigned kRowsBytes = 2u * MX * TY * (unsigned)MB + (unsigned)FX * TY * 4u;
  float v[kTmaStages][3][NP];
  MassElem<MR> m1[RS][NM], m2[RS][NM];
  float phi[RS][NF];
  unsigned long long bar[kTmaStages], mbar[RS];
};

__device__ __forceinline__ unsigned gbf_smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void gbf_mbar_init(unsigned long long* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(gbf_smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void gbf_mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void gbf_mbar_expect_tx(unsigned long long* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(gbf_smem_u32(b)), "r"(bytes) : "memory");
}
// Bounded wait for the completion of the barrier's phase `parity`.
__device__ __forceinline__ bool gbf_mbar_wait(unsigned long long* b, unsigned parity, unsigned max_tries) {
  for (unsigned it = 0; it < max_tries; ++it) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(gbf_smem_u32(b)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
// One plane box of a 3-D FP32 tensor into shared memory; the barrier
// receives the transferred bytes.
__device__ __forceinline__ void gbf_tma_plane(void* dst, const GbfTensorMap* map, int x, int y, int z,
                                              unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(gbf_smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(gbf_smem_u32(bar))
      : "memory");
}
// A try_wait round suspends the thread for up to about 3.8 us on GB300
// (measured with gbf_diag_bounded_wait), so a wait gives up after about 1 s
// and the drain of each copy still in flight after about 60 ms.
constexpr unsigned kTmaWaitTries = 1u << 18;   // a wait gives up after this many try_wait rounds
constexpr unsigned kTmaDrainTries = 1u << 14;  // after a give-up, per outstanding copy

// FP32 base-2 logarithm and exponential: the hardware approximations
// (PTX lg2.approx / ex2.approx, flush-to-zero; about 2^-22 relative error),
// ample for FP32 mobilities and capillary pressures.
__device__ __forceinline__ float split_lg2(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float split_ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// ----------------------------------------------------------- lane vectors
// The per-cell arithmetic below runs on N = 1 lane (float: the 32-wide tiles)
// or N = 2 lanes (float2: the two cells of an x-pair thread, on Blackwell's
// paired FP32 instructions, one instruction for both cells). Every operation
// is rounded explicitly (__fadd_rn, __fmul_rn, __fmaf_rn and their x2 forms,
// which round each lane as the scalar ones do), so that both widths give each
// cell the same bits. The assembler fuses a paired product that feeds a
// paired add into one paired FMA whatever the rounding suffix (measured on
// GB300), so the code below never lets a paired product (vmul) feed an add:
// a product and a sum are written as one explicit FMA (vfma, the same in
// both widths), and a product that must stay exactly rounded (a face flux
// carried to the next plane, the products of TwoSum) is taken lane by lane
// with the scalar __fmul_rn, which is never fused. Paired products feed
// multiplications, FMA operands and comparisons only.
template <int N> struct Lanes;
template <> struct Lanes<1> {
  using F = float;
  static __device__ __forceinline__ F splat(float x) { return x; }
  static __device__ __forceinline__ float get(F a, int) { return a; }
  template <class Fn> static __device__ __forceinline__ F make(Fn f) { return f(0); }
};
template <> struct Lanes<2> {
  using F = float2;
  static __device__ __forceinline__ F splat(float x) { return make_float2(x, x); }
  static __device__ __forceinline__ float get(F a, int n) { return n ? a.y : a.x; }
  template <class Fn> static __device__ __forceinline__ F make(Fn f) { return make_float2(f(0), f(1)); }
};
__device__ __forceinline__ float vadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float vneg(float a) { return -a; }
__device__ __forceinline__ float vabs(float a) { return fabsf(a); }
__device__ __forceinline__ float2 vneg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 vabs(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 vsub(float2 a, float2 b) { return __fadd2_rn(a, vneg(b)); }
__device__ __forceinline__ float2 vmul(float2 a, float2 b) { return __fmul2_rn(a, b); }
// Lane by lane exactly rounded products (never fused into a later add).
__device__ __forceinline__ float vmul_exact(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float2 vmul_exact(float2 a, float2 b) {
  return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// 1 / x (PTX rcp.approx, flush-to-zero; about 1 ulp).
__device__ __forceinline__ float split_rcp(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Mobility x density of both phases at one cell (FP32): Brooks-Corey kr
// (cpu.cpp:60-62) from one log2 and two exp2, Xi = -K kr / mu, densities at
// P2 = P1 (cpu.cpp:63, 72-73).
__device__ __forceinline__ void split_props(const GbfSplitConsts& C, int md, float K, float dP, float S, int j,
                                            float& L1, float& L2) {
  const float Pp = fmaf((float)j, C.H, dP);  // P - P_atm
  const float Se = fmaf(S, C.se_b[md], 1.f);  // (1 - S - S_wr) / (1 - S_wr)
  const float l2 = split_lg2(Se);
  const float kr1 = split_ex2(C.e1[md] * l2);
  const float om = 1.f - Se;
  const float kr2 = om * om * (1.f - split_ex2(C.e2[md] * l2));
  L1 = K * kr1 * C.nmr1 * fmaf(C.beta1, Pp, 1.f);  // nmr = -rho0 / mu
  L2 = K * kr2 * C.nmr2 * fmaf(C.beta2, Pp, 1.f);
}

// Upwinded flux through one face: the potential x (from the minus to the
// plus side) times the mobility of the cell the flow comes from, L_minus for
// x >= 0 and L_plus otherwise — the reference's ((x + |x|) L_minus + (x - |x|)
// L_plus) / 2 (cpu.cpp:260-262) — as one rounded product. A face's flux is
// then one value whichever of its two cells computes it: the two cells of a
// thread's pair share their middle x face, and the flux through the face
// above a plane is carried to the next plane as the flux through the face
// below it. In x and z both phases share the potential (P2 = P1), and so the
// comparison.
__device__ __forceinline__ float split_face(float x, float Lminus, float Lplus) {
  return __fmul_rn(x, x >= 0.f ? Lminus : Lplus);
}

// Brooks-Corey capillary pressure P_d S_e^(-1/lambda) and its S-derivative (cpu.cpp:303-308).
__device__ __forceinline__ float split_Pk(const GbfSplitConsts& C, int md, float S, float& dPk_dS) {
  const float Se = __fmaf_rn(S, C.se_b[md], 1.f);
  const float Pk = __fmul_rn(C.P_d[md], split_ex2(__fmul_rn(C.m_inv_lam[md], split_lg2(Se))));
  dPk_dS = __fmul_rn(__fmul_rn(Pk, C.inv_lam_1mswr[md]), split_rcp(Se));
  return Pk;
}

// A thread's sums over its cells: phase masses phi T (for the mass balance),
// largest CFL numbers, non-finite flag.
template <int MR>
struct GbfSplitAcc {  // kMassF64, kMassDF: phi T in the wide type
  using W = WideOf<MR>;
  typename W::T m1, m2;
  float cfl1, cfl2;  // largest CFL numbers of the thread's cells (when requested)
  unsigned bad;
  __device__ GbfSplitAcc() : m1(W::f(0.f)), m2(W::f(0.f)), cfl1(0.f), cfl2(0.f), bad(0) {}
  __device__ __forceinline__ void masses(double& a, double& b) const {
    a = W::tod(m1);
    b = W::tod(m2);
  }
};
// The FP32 defect form, per lane (.x: a thread's first cell, .y: the second
// cell of an x-pair thread): sum phi S as an FP32 pair, TwoSum (Knuth) into
// the high part with the exact errors (and those of the products phi S) in
// the low part, so that it keeps its relative precision however small it is
// (the DNAPL of the first steps); sum phi D1 and sum phi (D2 + rho02 beta2
// P_k S) in FP32 (small terms). c1, c2: the densities of the thread's row (a
// thread keeps one row j). The phase masses are -c1 sum phi S + sum phi D1
// (the grid's c1-weighted porosity sum, gbf_defect_k1, is added once per
// grid) and c2 sum phi S + sum phi (D2 + ...).
template <>
struct GbfSplitAcc<kMassDefect> {
  float2 sS, lS;  // per lane
  float b1, b2;   // both lanes
  float c1, c2;
  float cfl1, cfl2;
  unsigned bad;
  __device__ GbfSplitAcc()
      : sS{0.f, 0.f}, lS{0.f, 0.f}, b1(0.f), b2(0.f), c1(0.f), c2(0.f), cfl1(0.f), cfl2(0.f), bad(0) {}
  // phi = ph + pl (pl: the low part of a media-table porosity, has_pl)
  template <class F>
  static __device__ __forceinline__ void step(F& sS, F& lS, F ph, F pl, F S, bool has_pl) {
    const F p = vmul_exact(ph, S);  // TwoSum needs it rounded in every use
    F pe = vfma(ph, S, vneg(p));
    if (has_pl) pe = vfma(pl, S, pe);
    const F s = vadd(sS, p);
    const F bb = vsub(s, sS);
    lS = vadd(lS, vadd(vadd(vsub(sS, vsub(s, bb)), vsub(p, bb)), pe));
    sS = s;
  }
  __device__ __forceinline__ void add(float2 ph, float2 pl, float2 S, float2 D1, float2 D2q, bool has_pl) {
    step(sS, lS, ph, pl, S, has_pl);
    b1 = __fmaf_rn(ph.y, D1.y, __fmaf_rn(ph.x, D1.x, b1));
    b2 = __fmaf_rn(ph.y, D2q.y, __fmaf_rn(ph.x, D2q.x, b2));
  }
  __device__ __forceinline__ void add(float ph, float pl, float S, float D1, float D2q, bool has_pl) {
    step(sS.x, lS.x, ph, pl, S, has_pl);
    b1 = __fmaf_rn(ph, D1, b1);
    b2 = __fmaf_rn(ph, D2q, b2);
  }
  __device__ __forceinline__ void add_lane(int n, float ph, float pl, float S, float D1, float D2q, bool has_pl) {
    if (n)
      step(sS.y, lS.y, ph, pl, S, has_pl);
    else
      step(sS.x, lS.x, ph, pl, S, has_pl);
    b1 = __fmaf_rn(ph, D1, b1);
    b2 = __fmaf_rn(ph, D2q, b2);
  }
  __device__ __forceinline__ void masses(double& a, double& b) const {
    const double S = __dadd_rn(__dadd_rn((double)sS.x, (double)lS.x), __dadd_rn((double)sS.y, (double)lS.y));
    a = __dsub_rn((double)b1, __dmul_rn((double)c1, S));
    b = __dadd_rn(__dmul_rn((double)c2, S), (double)b2);
  }
};
// Pair defects: sum phi S, sum phi D1 and sum phi (D2 + q) as FP32 pairs
// (each product's rounding error kept, TwoSum into the high part; q = rho02
// beta2 P_k S, the DNAPL mass's small capillary term, joins D2 by one TwoSum,
// its error into the low part). pl: the low part of a media-table porosity
// (has_pl; zero with a porosity field, whose FP32 values are exact).
template <>
struct GbfSplitAcc<kMassDefectDF> {
  float sS, lS;
  GbfDF b1, b2;
  float c1, c2;
  float cfl1, cfl2;
  unsigned bad;
  __device__ GbfSplitAcc()
      : sS(0.f), lS(0.f), b1{0.f, 0.f}, b2{0.f, 0.f}, c1(0.f), c2(0.f), cfl1(0.f), cfl2(0.f), bad(0) {}
  __device__ __forceinline__ void add(float ph, float pl, float S, GbfDF D1, GbfDF D2, float q, bool has_pl) {
    const float p = __fmul_rn(ph, S);
    float pe = __fmaf_rn(ph, S, -p);
    if (has_pl) pe = __fmaf_rn(pl, S, pe);
    const float s = __fadd_rn(sS, p);
    const float bb = __fsub_rn(s, sS);
    lS = __fadd_rn(lS, __fadd_rn(__fadd_rn(__fsub_rn(sS, __fsub_rn(s, bb)), __fsub_rn(p, bb)), pe));
    sS = s;
    const GbfDF d2 = df_two_sum(D2.hi, q);  // D2 + q, not renormalised: acc_phi takes both parts
    const GbfDF D2q = {d2.hi, __fadd_rn(d2.lo, D2.lo)};
    b1 = Wide<true>::acc_phi(b1, ph, D1);
    b2 = Wide<true>::acc_phi(b2, ph, D2q);
    if (has_pl) {
      b1.lo = __fmaf_rn(pl, D1.hi, b1.lo);
      b2.lo = __fmaf_rn(pl, D2q.hi, b2.lo);
    }
  }
  __device__ __forceinline__ void masses(double& a, double& b) const {
    const double S = __dadd_rn((double)sS, (double)lS);
    a = __dsub_rn(Wide<true>::tod(b1), __dmul_rn((double)c1, S));
    b = __dadd_rn(__dmul_rn((double)c2, S), Wide<true>::tod(b2));
  }
};

// ------------------------------------------------------- one cell's update
// Inputs of one cell at plane k: the cell, its x and y neighbours (y = the
// vertical j), its column at plane k + 1, and both phases' fluxes through its
// face towards plane k - 1 (the previous plane's out-fluxes, split_face).
struct GbfCellIn {
  float dPc, S0, L1c, L2c;
  float dPxm, dPxp, dPym, dPyp;
  float L1xm, L1xp, L1ym, L1yp, L2xm, L2xp, L2ym, L2yp;
  float fz1, fz2;
  float dPp, L1p, L2p;
  float phi;
};
template <int MR>
struct GbfCellOut {
  float dPn, Sn;
  typename MassRep<MR>::T M1n, M2n;
  float fz1, fz2;  // fluxes through the face towards plane k + 1 (the next plane's fz1, fz2)
};
// Both phases' fluxes through the z face between a column's cells at planes
// k - 1 (dPm, L1m, L2m) and k: the carry a tile starts its first plane with.
__device__ __forceinline__ void split_zface(const GbfSplitConsts& C, float dPm, float L1m, float L2m, float dPc,
                                            float L1c, float L2c, float& fz1, float& fz2) {
  const float z = dPm - dPc;
  fz1 = split_face(z, L1m, L1c);
  fz2 = split_face(z, L2m, L2c);
}

// Flags of a thread's row and columns, fixed for a tile (the member
// constants are re-read from shared memory after every barrier, so the tile
// computes them once): bit 0 the no-flow bottom row (j = ny - 2 with
// GBF_BC_HYDROSTATIC_SIDES); bit 1 + n lane n's cell lies in the rate
// source's row and columns (j = 1, i in the patch).
template <int N>
__device__ __forceinline__ unsigned split_row_flags(const GbfSplitConsts& C, int j, const int (&ci)[N]) {
  unsigned f = (C.noflow_bottom && j == C.ny - 2) ? 1u : 0u;
#pragma unroll
  for (int n = 0; n < N; n++)
    if (j == 1 && ci[n] >= C.ri0 && ci[n] < C.ri0 + C.rn) f |= 2u << n;
  return f;
}

// The fused a3 + a4 update of N interior cells of one row and plane
// (cpu.cpp:218-320 in the split form): donor-cell fluxes, FP32 mass
// increments, mass targets (rate source added exactly), the residual, and the
// FP32 increment Newton. Wide forms: targets T = M + dm in the wide type, the
// residual split into its exact large part and FP32 small parts. Defect form:
// the residual and the new defects from FP32 operations on small numbers
// (rw: the row's densities). The arithmetic runs on lane vectors (Lanes<N>:
// one instruction for both cells of an x-pair thread where the two cells do
// the same operation) with explicit roundings, so that N = 1 and N = 2 give
// each cell the same bits; the x faces (a pair's middle face is one value),
// the upwind selections, the MUFU functions and the rare branches (rate
// source, second Newton iteration) run lane by lane. Lanes with count[n]
// false are computed but neither added to the mass sums nor checked for
// non-finite values. PATCH, for a grid with patch_in set: the source's cells
// are those under the Dirichlet patch, whose DNAPL inflow through the patch
// face comes in FP64 from the step's pre-pass (gbf_split_patch_cell) as
// patch_in[(i - ri0) + rn (k - rk0)] (i0 the column of lane 0) and takes the
// place of that face in the FP32 divergence. Grids without patch_in (an
// ensemble's rate-source members beside a patch member) keep the rate source
// in the PATCH tiles; the instantiations without PATCH, the tiles of every
// workload without a patch, have no patch code at all.
template <int MR, int N, bool CFL = false, bool PATCH = false>
__device__ __forceinline__ void split_cells(const GbfSplitConsts& C, const GbfCellIn (&in)[N],
                                            const typename MassRep<MR>::T (&M1)[N],
                                            const typename MassRep<MR>::T (&M2)[N], typename WideOf<MR>::T R01,
                                            typename WideOf<MR>::T R02, const GbfDefectRow& rw, int md,
                                            unsigned rowf, int j, int k, bool phi_field, bool mass,
                                            const bool (&count)[N], GbfSplitAcc<MR>& acc, GbfCellOut<MR> (&o)[N],
                                            const float2* patch_in, int i0) {
  using W = WideOf<MR>;
  using WT = typename W::T;
  using L = Lanes<N>;
  using F = typename L::F;
  constexpr bool DEF = gbf_is_defect(MR);
  const bool noflow = rowf & 1u;
  auto sp = [](float x) { return L::splat(x); };
  // the upwinded face flux of split_face on lane vectors
  // upwind mobility of a face with potential x (split_face), and the face
  // flux as a paired product (FMA operands only) or exactly rounded
  auto upw = [](F x, F Lm, F Lp) {
    return L::make([&](int n) { return L::get(x, n) >= 0.f ? L::get(Lm, n) : L::get(Lp, n); });
  };
  auto vface = [&](F x, F Lm, F Lp) { return vmul(x, upw(x, Lm, Lp)); };
  auto vface_exact = [&](F x, F Lm, F Lp) { return vmul_exact(x, upw(x, Lm, Lp)); };
  const F dPc = L::make([&](int n) { return in[n].dPc; });
  const F S0 = L::make([&](int n) { return in[n].S0; });
  const F L1c = L::make([&](int n) { return in[n].L1c; });
  const F L2c = L::make([&](int n) { return in[n].L2c; });
  // x faces lane by lane (the pair's middle face is one value for both
  // cells): flux differences in - out of both phases
  float ax1[N], ax2[N], bx1[N], bx2[N], dx1[N], dx2[N];
#pragma unroll
  for (int n = 0; n < N; n++) {
    const float x1 = __fsub_rn(in[n].dPxm, in[n].dPc), x2 = __fsub_rn(in[n].dPc, in[n].dPxp);
    ax1[n] = split_face(x1, in[n].L1xm, in[n].L1c);
    ax2[n] = split_face(x2, in[n].L1c, in[n].L1xp);
    bx1[n] = split_face(x1, in[n].L2xm, in[n].L2c);
    bx2[n] = split_face(x2, in[n].L2c, in[n].L2xp);
    dx1[n] = __fsub_rn(ax1[n], ax2[n]);
    dx2[n] = __fsub_rn(bx1[n], bx2[n]);
  }
  // y and z face potentials relative to the hydrostatic profile (P2 = P1),
  // times h: pressure differences, gravity terms scaled by h2
  const F Pp = vfma(sp((float)j), sp(C.H), dPc);  // P - P_atm
  const F gd2 = vfma(sp(C.gh2), Pp, sp(C.ghd));     // (rho2 - rho01) g h2
  const F yb1 = vsub(L::make([&](int n) { return in[n].dPym; }), dPc);
  const F yb2 = vsub(dPc, L::make([&](int n) { return in[n].dPyp; }));
  const F z2 = vsub(dPc, L::make([&](int n) { return in[n].dPp; }));
  // + (rho1 - rho01) g h2 = gh1 Pp
  const F y11 = vfma(sp(C.gh1), Pp, yb1), y12 = vadd(yb1, gd2);
  const F y21 = noflow ? sp(0.f) : vfma(sp(C.gh1), Pp, yb2), y22 = noflow ? sp(0.f) : vadd(yb2, gd2);
  // face fluxes, in through the minus face and out through the plus face:
  // the plus face's upwinded product, the minus face's inside the FMA of the
  // difference; the z face's out-flux exactly rounded (carried to the next
  // plane as its in-flux)
  const F L1ym = L::make([&](int n) { return in[n].L1ym; }), L2ym = L::make([&](int n) { return in[n].L2ym; });
  const F ay2 = vface(y21, L1c, L::make([&](int n) { return in[n].L1yp; }));
  const F by2 = vface(y22, L2c, L::make([&](int n) { return in[n].L2yp; }));
  const F az2 = vface_exact(z2, L1c, L::make([&](int n) { return in[n].L1p; }));
  const F bz2 = vface_exact(z2, L2c, L::make([&](int n) { return in[n].L2p; }));
  const F az1 = L::make([&](int n) { return in[n].fz1; });
  const F bz1 = L::make([&](int n) { return in[n].fz2; });
#pragma unroll
  for (int n = 0; n < N; n++) {
    o[n].fz1 = L::get(az2, n);
    o[n].fz2 = L::get(bz2, n);
  }
  const F dy1 = vfma(y11, upw(y11, L1ym, L1c), vneg(ay2));  // ay1 - ay2
  F dy2 = vfma(y12, upw(y12, L2ym, L2c), vneg(by2));
  bool patch = false;  // the source is the Dirichlet patch's FP64 inflow
  if constexpr (PATCH) {  // the patch face leaves the FP32 divergence (its FP64 inflow is the source below)
    patch = patch_in != nullptr;
    if (patch && (rowf >> 1) != 0u && (unsigned)(k - C.rk0) < (unsigned)C.rn)
      dy2 = L::make([&](int n) { return ((rowf >> (1 + n)) & 1u) ? -L::get(by2, n) : L::get(dy2, n); });
  }
  // dt times the flux divergence: sum over directions of (in - out) dt / h^2
  // (kv in y), then the FP32 mass increments -(..) / phi
  const F f = vfma(vsub(az1, az2), sp(C.wz),
                   vfma(dy1, sp(C.wy), vmul(L::make([&](int n) { return dx1[n]; }), sp(C.wx))));
  const F gs = vfma(vsub(bz1, bz2), sp(C.wz),
                    vfma(dy2, sp(C.wy), vmul(L::make([&](int n) { return dx2[n]; }), sp(C.wx))));
  const F nrphi = L::make([&](int n) { return split_rcp(-in[n].phi); });  // -1 / phi
  const F dm1 = vmul(f, nrphi), dm2 = vmul(gs, nrphi);  // FMA addends only
  if (CFL) {
#pragma unroll
    for (int n = 0; n < N; n++)
      if (count[n]) {
        // CFL number of each phase: the largest face volumetric flux of the
        // cell (mass flux x L_upwind over the reference density) times
        // dt / (phi h) (the mobilities L are <= 0: magnitudes by fabsf)
        const float ay1 = split_face(L::get(y11, n), in[n].L1ym, in[n].L1c);
        const float ay2n = split_face(L::get(y21, n), in[n].L1c, in[n].L1yp);
        const float by1 = split_face(L::get(y12, n), in[n].L2ym, in[n].L2c);
        const float by2n = split_face(L::get(y22, n), in[n].L2c, in[n].L2yp);
        const float c1 = fmaxf(fmaxf(__fmul_rn(fmaxf(fabsf(ax1[n]), fabsf(ax2[n])), C.wx),
                                     __fmul_rn(fmaxf(fabsf(ay1), fabsf(ay2n)), C.wy)),
                               __fmul_rn(fmaxf(fabsf(L::get(az1, n)), fabsf(L::get(az2, n))), C.wz));
        const float c2 = fmaxf(fmaxf(__fmul_rn(fmaxf(fabsf(bx1[n]), fabsf(bx2[n])), C.wx),
                                     __fmul_rn(fmaxf(fabsf(by1), fabsf(by2n)), C.wy)),
                               __fmul_rn(fmaxf(fabsf(L::get(bz1, n)), fabsf(L::get(bz2, n))), C.wz));
        const float rphi = -L::get(nrphi, n);
        acc.cfl1 = fmaxf(acc.cfl1, __fmul_rn(__fmul_rn(c1, rphi), C.cfl1));
        acc.cfl2 = fmaxf(acc.cfl2, __fmul_rn(__fmul_rn(c2, rphi), C.cfl2));
      }
  }
  WT T1[N], T2[N];
  if constexpr (!DEF) {  // mass targets T = M + dm (wide)
#pragma unroll
    for (int n = 0; n < N; n++) {
      T1[n] = W::add_f(M1[n], __fmul_rn(L::get(f, n), L::get(nrphi, n)));  // exactly rounded dm
      T2[n] = W::add_f(M2[n], __fmul_rn(L::get(gs, n), L::get(nrphi, n)));
    }
  }
  // the rate source, added exactly (defect form: its FP32 high and low parts)
  float srcf[N], srcl[N];
  bool insrc[N], anysrc = false;
  const bool ksrc = (rowf >> 1) != 0u && (unsigned)(k - C.rk0) < (unsigned)C.rn;
#pragma unroll
  for (int n = 0; n < N; n++) {
    srcf[n] = 0.f;
    srcl[n] = 0.f;
    insrc[n] = ksrc && ((rowf >> (1 + n)) & 1u);
    anysrc |= insrc[n];
  }
  if (patch) {  // the Dirichlet patch's FP64 inflow (an FP32 pair) in place of the rate (PATCH only)
    if (anysrc) {
#pragma unroll
      for (int n = 0; n < N; n++)
        if (insrc[n]) {  // i0 + n in [ri0, ri0 + rn), k in [rk0, rk0 + rn): inside the rn x rn array
          const float2 wp = patch_in[(i0 + n - C.ri0) + C.rn * (k - C.rk0)];
          if constexpr (DEF) {
            srcf[n] = wp.x;
            srcl[n] = wp.y;
          } else {
            T2[n] = W::add(T2[n], W::c((double)wp.x + (double)wp.y, wp));
            srcf[n] = wp.x;
          }
        }
    }
  } else if (anysrc) {
#pragma unroll
    for (int n = 0; n < N; n++) {
      const WT src = phi_field ? W::div_f(W::c(C.dtsrc_d, C.dtsrc_df), in[n].phi)
                               : W::c(C.dtsrc_m_d[md], C.dtsrc_m_df[md]);
      if constexpr (DEF) {
        if (insrc[n]) {
          srcf[n] = src.hi;
          srcl[n] = src.lo;
        }
      } else {
        const WT t2 = W::add(T2[n], src);
        if (insrc[n]) {
          T2[n] = t2;
          srcf[n] = W::tof(src);
        }
      }
    }
  }
  // residual r = F(P, S) - T at the stored state, cpu.cpp:305-306. Wide
  // forms: its large part rho0 (1 - S) - M (wide; the products of FP32
  // numbers are exact) and small FP32 parts rho0 beta P' (..) and dm:
  //   r1 = (rho01 - M1 - rho01 S) + rho01 beta1 P' (1 - S) - dm1
  //   r2 = (rho02 S - M2) + rho02 beta2 (P' + P_k) S - dm2 - src
  // Defect form (M1 = c1 (1 - S) + D1, M2 = c2 S + D2, c = rho0 (1 + beta j H) - e):
  //   r1 = (rho01 beta1 dP + e1) (1 - S) - D1 - dm1
  //   r2 = (rho02 beta2 (dP + P_k) + e2) S - D2 - dm2 - src
  // then the FP32 Newton on d = (dp, ds): r + [F(x + d) - F(x)] = 0, the
  // bracket written in increments so that no large terms cancel. The
  // equations are linear up to terms beta (dp ds, P_k'' ds^2): after the
  // first (linear) iteration the residual is about rho0 beta |dp ds|; a
  // second iteration runs when that could move S by more than 1e-9.
  // Capillary pressure P_d S_e^(-1/lambda) and its S-derivative (split_Pk).
  const F Se = vfma(S0, sp(C.se_b[md]), sp(1.f));
  const F lSe = L::make([&](int n) { return split_lg2(L::get(Se, n)); });
  const F exS = vmul(sp(C.m_inv_lam[md]), lSe);
  const F eS = L::make([&](int n) { return split_ex2(L::get(exS, n)); });
  const F Pk0 = vmul(sp(C.P_d[md]), eS);  // FMA operands only; its sums below are FMAs
  const F rSe0 = L::make([&](int n) { return split_rcp(L::get(Se, n)); });
  const F dPk0 = vmul(vmul(Pk0, sp(C.inv_lam_1mswr[md])), rSe0);
  const F PpPk = vfma(sp(C.P_d[md]), eS, Pp);  // P' + P_k
  const F omS = vsub(sp(1.f), S0);
  F r1, r2;
  if constexpr (DEF) {
    const F D1 = L::make([&](int n) { return defect_f(M1[n]); });
    const F D2 = L::make([&](int n) { return defect_f(M2[n]); });
    // - dm = + f / phi inside the FMA
    r1 = vfma(vneg(f), nrphi, vfma(vfma(sp(C.ro01b1), dPc, sp(rw.e1)), omS, vneg(D1)));
    r2 = vsub(vfma(vneg(gs), nrphi,
                   vfma(vfma(sp(C.ro02b2), vfma(sp(C.P_d[md]), eS, dPc), sp(rw.e2)), S0, vneg(D2))),
              L::make([&](int n) { return srcf[n]; }));
  } else {
    r1 = L::make([&](int n) {
      return __fmaf_rn(-L::get(f, n), L::get(nrphi, n),
                       __fmaf_rn(__fmul_rn(C.ro01b1, L::get(Pp, n)), L::get(omS, n),
                                 W::rho_1mS_minus(R01, M1[n], in[n].S0)));
    });
    r2 = L::make([&](int n) {
      return __fsub_rn(__fmaf_rn(-L::get(gs, n), L::get(nrphi, n),
                                 __fmaf_rn(__fmul_rn(C.ro02b2, L::get(PpPk, n)), in[n].S0,
                                           W::rhoS_minus(R02, M2[n], in[n].S0))),
                       srcf[n]);
    });
  }
  const F a0 = vfma(sp(C.beta1), Pp, sp(1.f));
  const F b0 = vfma(sp(C.beta2), PpPk, sp(1.f));
  const F J11 = vmul(sp(C.ro01b1), omS), mJ12 = vmul(sp(C.ro01), a0);  // J12 = -mJ12
  const F J21 = vmul(sp(C.ro02b2), S0), J22 = vmul(sp(C.ro02), vfma(vmul(sp(C.beta2), dPk0), S0, b0));
  const F ninv = L::make([&](int n) { return split_rcp(-L::get(vfma(J11, J22, vmul(mJ12, J21)), n)); });
  const F tp = vfma(J22, r1, vmul(mJ12, r2));       // J22 r1 - J12 r2
  const F ts = vfma(J11, r2, vneg(vmul(J21, r1)));  // J11 r2 - J21 r1
  const F dp = vmul(ninv, tp), ds = vmul(ninv, ts);  // the first step (FMA operands only)
  const F nl = vmul(vmul(sp(C.bmax), vabs(ds)), vadd(vfma(sp(4.f), vabs(vmul(dPk0, ds)), vabs(dp)), sp(1.f)));
  F Pk = vfma(dPk0, ds, Pk0);
  bool need[N], anyneed = false;
#pragma unroll
  for (int n = 0; n < N; n++) {
    need[n] = L::get(nl, n) > 1e-9f;
    anyneed |= need[n];
  }
  // the new state: the first step inside one FMA each
  F dPn = vfma(ninv, tp, dPc), Sn = vfma(ninv, ts, S0);
  // (the corrected form below takes its second step from the exact residual instead)
  if (MR != kMassDefectDF && anyneed) {
    float dpn[N], dsn[N], Pkn[N];
#pragma unroll
    for (int n = 0; n < N; n++) {
      // from the state the first step reached: its increments as applied
      const float s0 = in[n].S0, pk0 = __fmul_rn(C.P_d[md], L::get(eS, n));
      const float p = __fsub_rn(L::get(dPn, n), in[n].dPc), s = __fsub_rn(L::get(Sn, n), s0);
      // a0, b0 of this lane again (the same operations), not kept across the branch
      const float Ppn = __fmaf_rn((float)j, C.H, in[n].dPc);
      const float a = __fmaf_rn(C.beta1, Ppn, 1.f);
      const float b = __fmaf_rn(C.beta2, __fmaf_rn(C.P_d[md], L::get(eS, n), Ppn), 1.f);
      float dPk1;
      const float S1 = __fadd_rn(s0, s);
      const float Pk1 = split_Pk(C, md, S1, dPk1);
      const float dpk = __fadd_rn(p, __fsub_rn(Pk1, pk0));
      const float G1 =
          __fmaf_rn(C.ro01, __fmaf_rn(-a, s, __fmul_rn(__fmul_rn(C.beta1, p), __fsub_rn(1.f, S1))), L::get(r1, n));
      const float G2 = __fmaf_rn(C.ro02, __fmaf_rn(b, s, __fmul_rn(__fmul_rn(C.beta2, dpk), S1)), L::get(r2, n));
      const float K11 = __fmul_rn(C.ro01b1, __fsub_rn(1.f, S1));
      const float mK12 = __fmul_rn(C.ro01, __fmaf_rn(C.beta1, p, a));
      const float K21 = __fmul_rn(C.ro02b2, S1);
      const float K22 = __fmul_rn(C.ro02, __fmaf_rn(__fmul_rn(C.beta2, dPk1), S1, __fmaf_rn(C.beta2, dpk, b)));
      const float inv = split_rcp(__fmaf_rn(K11, K22, __fmul_rn(mK12, K21)));
      const float ep = __fmul_rn(inv, __fmaf_rn(K22, G1, __fmul_rn(mK12, G2)));
      const float es = __fmul_rn(inv, __fmaf_rn(K11, G2, -__fmul_rn(K21, G1)));
      dpn[n] = need[n] ? __fadd_rn(in[n].dPc, __fsub_rn(p, ep)) : L::get(dPn, n);
      dsn[n] = need[n] ? __fadd_rn(s0, __fsub_rn(s, es)) : L::get(Sn, n);
      // P_k at the final S, to first order in the last correction
      Pkn[n] = need[n] ? __fmaf_rn(-dPk1, es, Pk1) : L::get(Pk, n);
    }
    dPn = L::make([&](int n) { return dpn[n]; });
    Sn = L::make([&](int n) { return dsn[n]; });
    Pk = L::make([&](int n) { return Pkn[n]; });
  }
  if constexpr (MR == kMassDefectDF) {
    // One residual-correction Newton step per cell (iterative refinement),
    // the second step of this form's Newton: the nonlinear residual of both
    // mass equations at the state (p1, S1) the FP32 step reached, against the
    // step's targets held at FP64 precision (the pair defect plus this step's
    // increment: T1 - c1 (1 - S1) = D1 + dm1 + c1 (S1 - S0), T2 - c2 S1 =
    // D2 + dm2 + src - c2 (S1 - S0)), with the capillary pressure P_k(S1)
    // evaluated afresh (it is stiff near residual saturation, S_e -> 0):
    //   r1 = (rho01 beta1 p1 + e1) (1 - S1) - T1',  r2 = (rho02 beta2 (p1 + P_k(S1)) + e2) S1 - T2'.
    // Error-free transformations (TwoSum, FastTwoSum, TwoProduct through FMA:
    // Knuth, Dekker) keep every large term exact, so the residual rounds at
    // about 2^-24 of the small hydrostatic remainder e (6e-13 of a density,
    // near an FP64 mass's own rounding), where the FP32 step's residual rounds
    // at 2^-24 of the defects (of the masses themselves at compressibility
    // 1e-4). The Jacobian is taken at (p1, S1) too, with its own reciprocals
    // of S_e and of the determinant (a refinement of the first step's would
    // carry the square of their change over the step, 14% where 1 - S falls
    // by a third in one step near residual saturation, and leave the
    // correction that much short).
    // On lane vectors like the rest; products that feed a TwoSum or an add
    // are taken lane by lane (vmul_exact), never fused.
    auto two_sum = [](F a, F b, F& s, F& e) {
      s = vadd(a, b);
      const F bb = vsub(s, a);
      e = vadd(vsub(a, vsub(s, bb)), vsub(b, bb));
    };
    const F S1 = Sn, p1 = dPn;
    const F Se1 = vfma(S1, sp(C.se_b[md]), sp(1.f));
    const F lS1 = L::make([&](int n) { return split_lg2(L::get(Se1, n)); });
    const F ex1 = vmul(sp(C.m_inv_lam[md]), lS1);
    const F Pk1 = vmul_exact(sp(C.P_d[md]), L::make([&](int n) { return split_ex2(L::get(ex1, n)); }));
    // targets: T' = D + t as (hi, err) beside D's low part
    const F ds1 = vsub(S1, S0);
    const F t1 = vfma(sp(rw.c1), ds1, dm1);
    F t2 = vfma(sp(-rw.c2), ds1, dm2);
    if (anysrc)
      t2 = L::make([&](int n) {
        return insrc[n] ? __fadd_rn(__fmaf_rn(-rw.c2, L::get(ds1, n), srcf[n]),
                                    __fadd_rn(__fmul_rn(L::get(gs, n), L::get(nrphi, n)), srcl[n]))
                        : L::get(t2, n);
      });
    F T1h, T1e, T2h, T2e;
    two_sum(L::make([&](int n) { return M1[n].hi; }), t1, T1h, T1e);
    two_sum(L::make([&](int n) { return M2[n].hi; }), t2, T2h, T2e);
    const F T1l = vadd(T1e, L::make([&](int n) { return M1[n].lo; }));
    const F T2l = vadd(T2e, L::make([&](int n) { return M2[n].lo; }));
    // water: a1 = rho01 beta1 p1 exactly as a1 + a1e, B = 1 - S1 exactly as
    // Bh + Be (FastTwoSum, S1 <= 1); a1 Bh - T1' inside one FMA (a small
    // result), the small terms beside it
    const F a1 = vmul_exact(sp(C.ro01b1), p1);
    const F a1e = vfma(sp(C.ro01b1_lo), p1, vfma(sp(C.ro01b1), p1, vneg(a1)));
    const F Bh = vsub(sp(1.f), S1);
    const F Be = vsub(vsub(sp(1.f), Bh), S1);
    const F r1 = vadd(vfma(a1, Bh, vneg(T1h)), vfma(vadd(sp(rw.e1), a1e), Bh, vfma(a1, Be, vneg(T1l))));
    // DNAPL: q = p1 + P_k exactly as qh + qe, a2 = rho02 beta2 q exactly as a2 + a2e
    F qh, qe;
    two_sum(p1, Pk1, qh, qe);
    const F a2 = vmul_exact(sp(C.ro02b2), qh);
    const F a2e = vfma(sp(C.ro02b2), qe, vfma(sp(C.ro02b2_lo), qh, vfma(sp(C.ro02b2), qh, vneg(a2))));
    const F r2 = vadd(vfma(a2, S1, vneg(T2h)), vfma(vadd(sp(rw.e2), a2e), S1, vneg(T2l)));
    // One Newton step with the Jacobian at (p1, S1) where the first step
    // moved S by more than 1e-3 of S_e (which also bounds 1 - S), the
    // first step's elsewhere: there every entry of the Jacobian changed by
    // less than about 1e-3 over the step, so the step it gives is short by
    // that much of a correction that is itself small. Lane by lane, so that
    // each cell takes the same path in every tile shape.
    F K11 = J11, mK12 = mJ12, K21 = J21, K22 = J22, kinv = ninv, dPk1 = dPk0;
    bool fresh[N], anyfresh = false;
#pragma unroll
    for (int n = 0; n < N; n++) {
      fresh[n] = __fmul_rn(fabsf(L::get(ds1, n)), L::get(rSe0, n)) > 1e-3f;
      anyfresh |= fresh[n];
    }
    if (anyfresh) {
      const F rSe1 = L::make([&](int n) { return split_rcp(L::get(Se1, n)); });  // 1 / S_e(S1)
      const F Pp1 = vfma(sp((float)j), sp(C.H), p1);
      const F dPkf = vmul(vmul(Pk1, sp(C.inv_lam_1mswr[md])), rSe1);
      const F K11f = vmul(sp(C.ro01b1), Bh), mK12f = vmul(sp(C.ro01), vfma(sp(C.beta1), Pp1, sp(1.f)));
      const F K21f = vmul(sp(C.ro02b2), S1);
      const F K22f =
          vmul(sp(C.ro02), vfma(vmul(sp(C.beta2), dPkf), S1, vfma(sp(C.beta2), vadd(Pp1, Pk1), sp(1.f))));
      const F kinvf = L::make([&](int n) { return split_rcp(-L::get(vfma(K11f, K22f, vmul(mK12f, K21f)), n)); });
      auto pick = [&](F a, F b) { return L::make([&](int n) { return fresh[n] ? L::get(a, n) : L::get(b, n); }); };
      K11 = pick(K11f, K11);
      mK12 = pick(mK12f, mK12);
      K21 = pick(K21f, K21);
      K22 = pick(K22f, K22);
      kinv = pick(kinvf, kinv);
      dPk1 = pick(dPkf, dPk1);
    }
    const F es = vmul(kinv, vfma(K11, r2, vneg(vmul(K21, r1))));
    dPn = vfma(kinv, vfma(K22, r1, vmul(mK12, r2)), p1);
    Sn = vadd(S1, es);
    Pk = vfma(dPk1, es, Pk1);  // P_k at the final S, to first order in the correction
  }
  const F fin = vadd(dPn, Sn);  // NaN and infinities carry through the sum
#pragma unroll
  for (int n = 0; n < N; n++) {
    o[n].dPn = L::get(dPn, n);
    o[n].Sn = L::get(Sn, n);
    if (count[n] && !isfinite(L::get(fin, n))) acc.bad = 1;
  }
  if constexpr (DEF) {
    // new defects: D1 + dm1 + c1 dS and D2 + dm2 + src - c2 dS - rho02 beta2 P_k S,
    // with dS the stored change of S and c dS against the increment it
    // balances inside one FMA (exact product, one rounding of a small sum)
    const F dse = vsub(Sn, S0);
    // q = rho02 beta2 P_k S: next step's ro2 S2 is taken without P_k
    // (cpu.cpp:63 vs :306); qa S inside the FMAs that subtract or add it
    const F qa = vmul(sp(C.ro02b2), Pk);
    const F i1 = vfma(sp(rw.c1), dse, dm1);
    F u = vfma(sp(-rw.c2), dse, dm2);
    if (anysrc)
      u = L::make([&](int n) {
        return insrc[n] ? __fadd_rn(__fmaf_rn(-rw.c2, L::get(dse, n), srcf[n]),
                                    __fadd_rn(__fmul_rn(L::get(gs, n), L::get(nrphi, n)), srcl[n]))
                        : L::get(u, n);
      });
    const F i2 = vfma(vneg(qa), Sn, u);  // u - q
    if constexpr (MR == kMassDefect) {
      const F D1n = vadd(L::make([&](int n) { return M1[n]; }), i1);
      const F D2n = vadd(L::make([&](int n) { return M2[n]; }), i2);
#pragma unroll
      for (int n = 0; n < N; n++) {
        o[n].M1n = L::get(D1n, n);
        o[n].M2n = L::get(D2n, n);
      }
      if (mass) {  // phi T with T1 = c1 (1 - S) + D1, T2 = c2 S + D2 + q
        const F ph = phi_field ? L::make([&](int n) { return in[n].phi; }) : sp(C.m_df[md].x);
        const F pl = sp(phi_field ? 0.f : C.m_df[md].y);
        bool all = true;
#pragma unroll
        for (int n = 0; n < N; n++) all = all && count[n];
        if (all)
          acc.add(ph, pl, Sn, D1n, vfma(qa, Sn, D2n), !phi_field);
        else
#pragma unroll
          for (int n = 0; n < N; n++)
            if (count[n])
              acc.add_lane(n, L::get(ph, n), L::get(pl, n), L::get(Sn, n), L::get(D1n, n),
                           __fmaf_rn(L::get(qa, n), L::get(Sn, n), L::get(D2n, n)), !phi_field);
      }
    } else {
#pragma unroll
      for (int n = 0; n < N; n++) {
        o[n].M1n = defect_add(M1[n], L::get(i1, n));
        o[n].M2n = defect_add(M2[n], L::get(i2, n));
        if (count[n] && mass) {
          const float ph = phi_field ? in[n].phi : C.m_df[md].x;
          const float pl = phi_field ? 0.f : C.m_df[md].y;
          acc.add(ph, pl, o[n].Sn, o[n].M1n, o[n].M2n, __fmul_rn(L::get(qa, n), o[n].Sn), !phi_field);
        }
      }
    }
  } else {
#pragma unroll
    for (int n = 0; n < N; n++) {
      o[n].M1n = T1[n];
      // next step's ro2 S2 is taken at P2 = P1, without P_k (cpu.cpp:63 vs :306)
      o[n].M2n = W::add_f(T2[n], __fmul_rn(__fmul_rn(-C.ro02b2, L::get(Pk, n)), o[n].Sn));
      if (count[n] && mass) {  // phi T in the wide type (phi exact: an FP32 input or a wide table value)
        if (phi_field) {
          acc.m1 = W::acc_phi(acc.m1, in[n].phi, T1[n]);
          acc.m2 = W::acc_phi(acc.m2, in[n].phi, T2[n]);
        } else {
          const WT phw = W::c(C.m_d[md], C.m_df[md]);
          acc.m1 = W::add(acc.m1, W::mul(phw, T1[n]));
          acc.m2 = W::add(acc.m2, W::mul(phw, T2[n]));
        }
      }
    }
  }
}

// One CTA: interior cells [i0, i0+TX) x [j0, j0+TY) of planes [k0, k1); i0,
// j0, k0 >= 1. `pl` points to two planes of shared memory.
//
// TMA = true: halo planes (dP, S of the state buffer `buf`, K) and interior
// rows (M1, M2, phi) arrive by cp.async.bulk.tensor into the rings of `raw`
// (a K and a phi field, no media table); `pl` holds three plane buffers. The
// call returns false if a bounded wait gave up (the status word then carries
// GBF_DEV_TIMEOUT). `phases` holds the barrier parities across calls.
// TMA = false: plain loads, one plane prefetched in registers, two buffers.
template <int MR, int TX = kSplitTX, int TY = kSplitTY, bool TMA = false, bool CFL = false, bool PATCH = false>
__device__ bool split_tile(const GbfSplitConsts& C, const GbfSplitGrid& G, int i0, int j0, int k0, int k1,
                           GbfSplitPlaneT<TX, TY, gbf_plane_pitch<TX, TMA>()>* pl, GbfSplitAcc<MR>& acc,
                           GbfRawRing<TX, TY, MR>* raw = nullptr, const GbfTmaSet* maps = nullptr, int buf = 0,
                           unsigned* phases = nullptr) {
  using W = WideOf<MR>;
  using WT = typename W::T;
  using MT = typename MassRep<MR>::T;
  constexpr int PX = gbf_plane_pitch<TX, TMA>();
  using Sh = GbfSplitShape<TX, TY, PX>;
  constexpr int kSplitTX = TX, kSplitThreads = Sh::threads, kSplitHX = Sh::HX, kSplitHN = Sh::HN,
                kSplitSlots = Sh::slots;
  using GbfSplitPlane = GbfSplitPlaneT<TX, TY, PX>;
  static_assert(!TMA || PX == GbfRawRing<TX, TY, MR>::BX, "TMA plane pitch equals the box width");
  const int nx = C.nx, ny = C.ny, nz = C.nz;
  const unsigned pln = (unsigned)nx * (unsigned)ny;  // grids hold < 2^32 cells (checked on the host)
  const int tx = threadIdx.x % kSplitTX, ty = threadIdx.x / kSplitTX;
  const int i = i0 + tx, j = j0 + ty;
  const bool active = (i <= nx - 2) && (j <= ny - 2);
  const int hc = (ty + 1) * kSplitHX + (tx + 1);  // own cell in the halo plane

  // halo elements of this thread: plane index, global column offset (or -1), row j
  int hq[kSplitSlots], hj[kSplitSlots];
  int hcol[kSplitSlots];
#pragma unroll
  for (int s = 0; s < kSplitSlots; s++) {
    const int q = threadIdx.x + s * kSplitThreads;
    hq[s] = q;
    hcol[s] = -1;
    hj[s] = 0;
    if (q < kSplitHN && q % kSplitHX < TX + 2) {
      const int gi = i0 - 1 + q % kSplitHX, gj = j0 - 1 + q / kSplitHX;
      if (gi < nx && gj < ny) {
        hcol[s] = gi + gj * nx;
        hj[s] = gj;
      }
    }
  }
  // raw inputs of the next plane, prefetched one plane ahead
  float rP[kSplitSlots], rS[kSplitSlots], rK[kSplitSlots];
  int rM[kSplitSlots];
  auto fetch = [&](int k) {
#pragma unroll
    for (int s = 0; s < kSplitSlots; s++) {
      rP[s] = 0.f; rS[s] = 0.f; rK[s] = 0.f; rM[s] = 0;
      if (hcol[s] >= 0 && k < nz) {
        const unsigned c = (unsigned)hcol[s] + (unsigned)k * pln;
        rP[s] = __ldg(G.dP + c);
        rS[s] = __ldg(G.S + c);
        rM[s] = G.media ? __ldg(G.media + c) : 0;
        rK[s] = G.K ? __ldg(G.K + c) : C.K[rM[s]];
      }
    }
  };
  auto build = [&](GbfSplitPlane& P) {
#pragma unroll
    for (int s = 0; s < kSplitSlots; s++) {
      if (hcol[s] >= 0) {
        float L1, L2;
        split_props(C, rM[s], rK[s], rP[s], rS[s], hj[s], L1, L2);
        P.dP[hq[s]] = rP[s];
        P.S[hq[s]] = rS[s];
        P.L1[hq[s]] = L1;
        P.L2[hq[s]] = L2;
      }
    }
  };

  // TMA staging. Plane p uses stage (p - k0) % kTmaStages of the halo ring,
  // stage (p - k0) % RS of the rows ring and plane buffer pl[(p - k0) % 3];
  // planes are issued and consumed in order, so each ring keeps rotating
  // issue and use counters instead. Thread 0 issues the copies; every thread
  // tracks the stages in flight (`pend`: bits 0.. halo ring, bits 8.. rows
  // ring) and the barrier parities (`*phases`, same bit layout), so that a
  // give-up can wait out the copies still in flight.
  using Ring = GbfRawRing<TX, TY, MR>;
  constexpr int RS = Ring::RS;
  unsigned pend = 0;
  int h_issue = 0, r_issue = 0;  // next stage to fill, halo and rows rings
  auto issue = [&](int p) {  // halo planes of plane p
    if constexpr (TMA) {
      const int s = h_issue;
      h_issue = s == kTmaStages - 1 ? 0 : s + 1;
      if (threadIdx.x == 0) {
        gbf_mbar_expect_tx(&raw->bar[s], Ring::kHaloBytes);
        gbf_tma_plane(raw->v[s][0], &maps->dP[buf], i0 - 1, j0 - 1, p, &raw->bar[s]);
        gbf_tma_plane(raw->v[s][1], &maps->S[buf], i0 - 1, j0 - 1, p, &raw->bar[s]);
        gbf_tma_plane(raw->v[s][2], &maps->K, i0 - 1, j0 - 1, p, &raw->bar[s]);
      }
      pend |= 1u << s;
    }
  };
  auto issue_rows = [&](int p) {  // M1, M2, phi rows of plane p
    if constexpr (TMA) {
      const int s = r_issue;
      r_issue = s == RS - 1 ? 0 : s + 1;
      if (threadIdx.x == 0) {
        gbf_mbar_expect_tx(&raw->mbar[s], Ring::kRowsBytes);
        gbf_tma_plane(raw->m1[s], &maps->M1, i0 - 1, j0, p, &raw->mbar[s]);
        gbf_tma_plane(raw->m2[s], &maps->M2, i0 - 1, j0, p, &raw->mbar[s]);
        gbf_tma_plane(raw->phi[s], &maps->phi, i0 - 1, j0, p, &raw->mbar[s]);
      }
      pend |= 1u << (8 + s);
    }
  };
  auto wait_bit = [&](int bit) -> bool {  // bounded wait for the stage of `bit`
    if constexpr (TMA) {
      unsigned long long* b = bit < 8 ? &raw->bar[bit] : &raw->mbar[bit - 8];
      if (!gbf_mbar_wait(b, (*phases >> bit) & 1u, kTmaWaitTries)) return false;
      *phases ^= 1u << bit;
      pend &= ~(1u << bit);
    }
    return true;
  };
  auto give_up = [&]() {  // after a wait gave up somewhere in the CTA
    if constexpr (TMA) {
      for (int bit = 0; bit < 16; bit++)
        if ((pend >> bit) & 1u) {
          unsigned long long* b = bit < 8 ? &raw->bar[bit] : &raw->mbar[bit - 8];
          gbf_mbar_wait(b, (*phases >> bit) & 1u, kTmaDrainTries);
          *phases ^= 1u << bit;
        }
      pend = 0;
      if (threadIdx.x == 0) atomicOr(G.status, GBF_DEV_TIMEOUT);
    }
  };
  auto build_tma = [&](GbfSplitPlane& P, int s) {  // from halo stage s
    if constexpr (TMA) {
#pragma unroll
      for (int q = 0; q < kSplitSlots; q++) {
        if (hcol[q] >= 0) {
          const int ri = hq[q];  // same pitch in the box and in the plane
          float L1, L2;
          const float rp = raw->v[s][0][ri], rs = raw->v[s][1][ri];
          split_props(C, 0, raw->v[s][2][ri], rp, rs, hj[q], L1, L2);
          P.dP[hq[q]] = rp;
          P.S[hq[q]] = rs;
          P.L1[hq[q]] = L1;
          P.L2[hq[q]] = L2;
        }
      }
    }
  };

  // prologue: own column at k0 - 1 (registers), plane k0 (shared)
  if constexpr (TMA) {
    for (int q = 0; q < kTmaStages && k0 + q <= k1; q++) issue(k0 + q);
    for (int q = 0; q < RS && k0 + q < k1; q++) issue_rows(k0 + q);
  }
  float dPm = 0.f, L1m = 0.f, L2m = 0.f;
  if (active) {
    const unsigned c = (unsigned)(i + j * nx) + (unsigned)(k0 - 1) * pln;
    const int md = G.media ? G.media[c] : 0;
    const float Kc = G.K ? G.K[c] : C.K[md];
    dPm = G.dP[c];
    split_props(C, md, Kc, dPm, G.S[c], j, L1m, L2m);
  }
  if constexpr (TMA) {
    const bool ok = wait_bit(0);
    if (ok) build_tma(pl[0], 0);
    if (__syncthreads_or(!ok)) {
      give_up();
      return false;
    }
    if (k0 + kTmaStages <= k1) issue(k0 + kTmaStages);
  } else {
    fetch(k0);
    build(pl[0]);
    fetch(k0 + 1);
    __syncthreads();
  }
  // flux carry: both phases through the face between planes k0 - 1 and k0
  float fz1 = 0.f, fz2 = 0.f;
  if (active) split_zface(C, dPm, L1m, L2m, pl[0].dP[hc], pl[0].L1[hc], pl[0].L2[hc], fz1, fz2);
  int cur = 0;                             // plain loads: buffer of plane k
  int t_cur = 0, t_next = 1, t_rows = 0;   // TMA: buffer/halo stage of planes k, k + 1; rows stage of plane k
  const WT R01 = W::c(C.ro01_d, C.ro01_df), R02 = W::c(C.ro02_d, C.ro02_df);
  const GbfDefectRow rw = gbf_is_defect(MR) ? gbf_defect_row(C, j) : GbfDefectRow{};
  const int cols[1] = {i};
  const unsigned rowf = split_row_flags<1>(C, j, cols);
  if constexpr (gbf_is_defect(MR)) {
    acc.c1 = rw.c1;
    acc.c2 = rw.c2;
  }
  const int mi = ty * Ring::MX + tx + 1, fi = ty * Ring::FX + tx + 1;  // own cell in the rows boxes
  for (int k = k0; k < k1; k++) {
    if constexpr (TMA) {
      // one barrier per plane: plane k + 1 built into its own buffer (three
      // buffers rotate, so no thread can still be reading the one written)
      const int sn = t_next;
      bool ok = wait_bit(sn);
      ok = ok && wait_bit(8 + t_rows);
      if (ok) build_tma(pl[sn], sn);
      if (__syncthreads_or(!ok)) {
        give_up();
        return false;
      }
      // halo stage sn was consumed by the build above; the rows stage of
      // plane k - 1 (= that of plane k - 1 + RS) by the previous plane's update
      if (k + 1 + kTmaStages <= k1) issue(k + 1 + kTmaStages);
      if (k > k0 && k - 1 + RS < k1) issue_rows(k - 1 + RS);
    } else {
      build(pl[cur ^ 1]);  // plane k + 1 from the prefetched raw values
      fetch(k + 2);        // prefetch plane k + 2
      __syncthreads();
    }
    GbfSplitPlane& Pc = TMA ? pl[t_cur] : pl[cur];
    GbfSplitPlane& Pn = TMA ? pl[t_next] : pl[cur ^ 1];
    const int sr = t_rows;
    if (active) {
      const unsigned c = (unsigned)(i + j * nx) + (unsigned)k * pln;
      const int md = (!TMA && G.media) ? __ldg(G.media + c) : 0;
      const float phi = TMA ? raw->phi[sr][fi] : (G.phi ? __ldg(G.phi + c) : C.m[md]);
      const MT M1 = TMA ? MassRep<MR>::load(reinterpret_cast<const double*>(raw->m1[sr]), mi)
                        : MassRep<MR>::load(G.M1, c);
      const MT M2 = TMA ? MassRep<MR>::load(reinterpret_cast<const double*>(raw->m2[sr]), mi)
                        : MassRep<MR>::load(G.M2, c);
      GbfCellIn in;
      in.dPc = Pc.dP[hc]; in.S0 = Pc.S[hc]; in.L1c = Pc.L1[hc]; in.L2c = Pc.L2[hc];
      in.dPxm = Pc.dP[hc - 1]; in.dPxp = Pc.dP[hc + 1];
      in.dPym = Pc.dP[hc - kSplitHX]; in.dPyp = Pc.dP[hc + kSplitHX];
      in.L1xm = Pc.L1[hc - 1]; in.L1xp = Pc.L1[hc + 1]; in.L1ym = Pc.L1[hc - kSplitHX]; in.L1yp = Pc.L1[hc + kSplitHX];
      in.L2xm = Pc.L2[hc - 1]; in.L2xp = Pc.L2[hc + 1]; in.L2ym = Pc.L2[hc - kSplitHX]; in.L2yp = Pc.L2[hc + kSplitHX];
      in.fz1 = fz1; in.fz2 = fz2;
      in.dPp = Pn.dP[hc]; in.L1p = Pn.L1[hc]; in.L2p = Pn.L2[hc];
      in.phi = phi;
      const GbfCellIn ins[1] = {in};
      const MT m1s[1] = {M1}, m2s[1] = {M2};
      const bool cnt[1] = {true};
      GbfCellOut<MR> os[1];
      split_cells<MR, 1, CFL, PATCH>(C, ins, m1s, m2s, R01, R02, rw, md, rowf, j, k, G.phi != nullptr,
                                     G.mass_partials != nullptr, cnt, acc, os, G.patch_in, i);
      G.dPn[c] = os[0].dPn;
      G.Sn[c] = os[0].Sn;
      MassRep<MR>::store(G.M1, c, os[0].M1n);
      MassRep<MR>::store(G.M2, c, os[0].M2n);
      fz1 = os[0].fz1;
      fz2 = os[0].fz2;
    }
    if constexpr (!TMA) {
      __syncthreads();
      cur ^= 1;
    } else {
      t_cur = t_next;
      t_next = t_next == kTmaStages - 1 ? 0 : t_next + 1;
      t_rows = t_rows == RS - 1 ? 0 : t_rows + 1;
    }
  }
  return true;
}

// Split state of one cell from FP64 P, S: dP = P - P_hs(j), S in FP32 and
// the phase masses ro1 (1 - S2), ro2 S2 with P2 = P1 (cpu.cpp:72-73, 224-225)
// in the representation `mr` (defect form: minus c1 (1 - S), c2 S of the
// FP32 S, products that are exact in FP64).
// A row's constants for the state conversions (GbfRowConst), as
// gbf_p_hydrostatic and gbf_defect_row give them.
__device__ __forceinline__ GbfRowConst gbf_row_const(const gbf_model& m, int j) {
  const GbfDefectRow w = gbf_defect_row(m, j);
  return {gbf_p_hydrostatic(m, j), w.c1, w.c2};
}
__device__ __forceinline__ void gbf_split_init_cell(const gbf_model& m, double p, double s, const GbfRowConst& rc,
                                                    float& dPf, float& Sf, double* M1, double* M2, size_t c, int mr) {
  dPf = (float)(p - rc.phs);
  Sf = (float)s;
  const double m1 = m.ro01 * (1. + m.beta1 * (p - m.P_atm)) * (1. - s);
  const double m2 = m.ro02 * (1. + m.beta2 * (p - m.P_atm)) * s;
  if (mr == kMassDefect) {
    reinterpret_cast<float*>(M1)[c] = (float)(m1 - (double)rc.c1 * (1. - (double)Sf));
    reinterpret_cast<float*>(M2)[c] = (float)(m2 - (double)rc.c2 * (double)Sf);
  } else if (mr == kMassDefectDF) {
    reinterpret_cast<float2*>(M1)[c] = gbf_df_from_double(m1 - (double)rc.c1 * (1. - (double)Sf));
    reinterpret_cast<float2*>(M2)[c] = gbf_df_from_double(m2 - (double)rc.c2 * (double)Sf);
  } else if (mr == kMassDF) {
    reinterpret_cast<float2*>(M1)[c] = gbf_df_from_double(m1);
    reinterpret_cast<float2*>(M2)[c] = gbf_df_from_double(m2);
  } else {
    M1[c] = m1;
    M2[c] = m2;
  }
}
__device__ __forceinline__ void gbf_split_init_cell(const gbf_model& m, double p, double s, int j, float& dPf,
                                                    float& Sf, double* M1, double* M2, size_t c, int mr) {
  gbf_split_init_cell(m, p, s, gbf_row_const(m, j), dPf, Sf, M1, M2, c, mr);
}

// Value the reference's boundary sweep leaves in P1 (cpu.cpp:366-403), in
// the dP = P - P_hs(j) representation: copies within a row keep dP, the top
// (P_atm) and the hydrostatic sides (P_hs) are dP = 0, and the bottom rule
// P(ny-1) = P(ny-2) + ro1(i,1,0) g h2 becomes dP(ny-2) + (ro1(i,1,0) - rho01) g h2.
__device__ __forceinline__ float gbf_split_sweep_dP(const gbf_model& m, const GbfGeo& g, const float* cur,
                                                    const float* old, int i, int j, int k, float H) {
  bool has_add = false;
  float add = 0.f, base = NAN;
  for (int hop = 0; hop < 6; ++hop) {
    if (m.bc_mode == GBF_BC_HYDROSTATIC_SIDES && (i == 0 || i == g.nx - 1 || k == 0 || k == g.nz - 1)) {
      base = 0.f;
      break;
    }
    if (i == 0) { base = gbf_later(g, cur, old, 1, j, k); break; }
    if (i == g.nx - 1) {
      i = g.nx - 2;
      if (!gbf_is_boundary(g, i, j, k)) { base = cur[gbf_idx(g, i, j, k)]; break; }
      continue;
    }
    if (j == g.ny - 1) {
      // start-of-step water density at (i, 1, 0): P - P_atm = dP_old + H
      const float pp = old[(size_t)i + (size_t)g.nx] + H;
      add = (float)(m.ro01 * m.beta1 * m.g * m.h2) * pp;
      has_add = true;
      j = g.ny - 2;
      if (!gbf_is_boundary(g, i, j, k)) { base = cur[gbf_idx(g, i, j, k)]; break; }
      continue;
    }
    if (j == 0) { base = 0.f; break; }
    if (k == 0) { base = gbf_later(g, cur, old, i, j, 1); break; }
    if (k == g.nz - 1) {
      k = g.nz - 2;
      if (!gbf_is_boundary(g, i, j, k)) { base = cur[gbf_idx(g, i, j, k)]; break; }
      continue;
    }
    base = cur[gbf_idx(g, i, j, k)];
    break;
  }
  return has_add ? base + add : base;
}

// One row segment of the face pass after the x-pair tile: a warp writes the
// new S and dP of cells i0 .. i0 + kFaceSeg - 1 (those below nx) of face row
// (j, k) (gbf_face_row), kFaceRound a lane. The rules read interior cells of
// the new state and boundary cells of the previous one, never a cell that
// this pass writes, so every value is read before any is written: a lane's
// loads are in flight together. j and k are the same for the whole warp, so
// only the row's end cells branch apart.
constexpr int kFaceRound = 4, kFaceSeg = 32 * kFaceRound;
__device__ __forceinline__ void gbf_split_face_segment(const gbf_model& m, const GbfGeo& g, const float* dP,
                                                       const float* S, float* dPn, float* Sn, float H, int j, int k,
                                                       int i0, int lane) {
  float sv[kFaceRound], pv[kFaceRound];
#pragma unroll
  for (int u = 0; u < kFaceRound; u++) {
    const int i = i0 + lane + 32 * u;
    sv[u] = pv[u] = 0.f;
    if (i < g.nx) {
      sv[u] = gbf_sweep_S<float>(m, g, Sn, S, i, j, k);
      pv[u] = gbf_split_sweep_dP(m, g, dPn, dP, i, j, k, H);
    }
  }
  const size_t row = gbf_idx(g, 0, j, k);
#pragma unroll
  for (int u = 0; u < kFaceRound; u++) {
    const int i = i0 + lane + 32 * u;
    if (i < g.nx) {
      Sn[row + i] = sv[u];
      dPn[row + i] = pv[u];
    }
  }
}

// Block maximum of the threads' CFL numbers (warp shuffles, then one thread
// over the warps' maxima), max-combined into out[2] with atomicMax on the
// bit patterns (non-negative floats order like their bits; NaN left out).
// Every thread of the block calls it.
template <int NT>
__device__ __forceinline__ void split_block_cfl(float c1, float c2, float* out) {
  __shared__ float red[2][NT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    c1 = fmaxf(c1, __shfl_xor_sync(0xffffffffu, c1, o));
    c2 = fmaxf(c2, __shfl_xor_sync(0xffffffffu, c2, o));
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][w] = c1; red[1][w] = c2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    float a = 0.f, b = 0.f;
    for (int q = 0; q < NT / 32; q++) { a = fmaxf(a, red[0][q]); b = fmaxf(b, red[1][q]); }
    atomicMax(reinterpret_cast<unsigned*>(out), __float_as_uint(a));
    atomicMax(reinterpret_cast<unsigned*>(out) + 1, __float_as_uint(b));
  }
  __syncthreads();  // red is reused by the next tile of a persistent CTA
}

// Deterministic block reduction of the threads' phase masses (FP64).
template <int NT>
__device__ __forceinline__ void split_block_mass_d(double a, double b, double V, double* out2) {
  __shared__ double red[2][NT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][w] = a; red[1][w] = b; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0., y = 0.;
    for (int q = 0; q < NT / 32; q++) { x += red[0][q]; y += red[1][q]; }
    out2[0] = x * V;
    out2[1] = y * V;
  }
}
template <int MR, int NT = kSplitThreads>
__device__ __forceinline__ void split_block_mass(const GbfSplitAcc<MR>& acc, double V, double* out2) {
  double a, b;
  acc.masses(a, b);
  split_block_mass_d<NT>(a, b, V, out2);
}

// ------------------------------------------------ x-pair tile (TMA only)
// A CTA of (TXC / 2) x TY threads owns TXC x TY cells; each thread updates the
// two cells x0 + 2 tx, x0 + 2 tx + 1 of row j0 + ty (tiles start at
// x0 = TXC * t, a multiple of 16 bytes). The halo box of a plane starts at
// x0 - 4 (16-byte aligned, zeros left of the grid) and is TXC + 8 wide, so a
// thread's pair sits at an even offset: its x-stencil is three 64-bit
// shared loads, its y neighbours and the plane above two more per field.
// The interior rows of M1, M2 and phi arrive as {TXC, TY} boxes at x0 (no
// halo), two planes ahead of the plane being updated (a 3-stage ring). The
// built planes hold dP, L1 and L2 of every box cell; S is needed only at the
// thread's own pair, which the thread builds itself and keeps in registers.
// Shared memory exceeds the static 48 KB, so the kernel takes it as dynamic
// shared memory (GbfPairSmem).
// Resident 256-thread x-pair CTAs per SM: three for the defect form (80
// registers a thread, 71 KB of shared memory), two for the wide forms
// (116-120 registers).
__host__ __device__ constexpr int gbf_pair_ctas(int MR) { return MR == kMassDefect ? 3 : 2; }

template <int TXC, int TY, int MR = kMassF64>
struct GbfPairRing {
  static_assert(TXC % 16 == 0 && TXC <= 248, "x-pair tile width");
  static constexpr int BX = TXC + 8, HY = TY + 2, N = BX * HY, NP = (N + 31) / 32 * 32;
  static constexpr int NR = TXC * TY;  // interior-row elements per field
  static constexpr int RS = 3;
  static constexpr unsigned MB = (unsigned)sizeof(MassElem<MR>);
  static constexpr unsigned kHaloBytes = 3u * N * 4u;
  static constexpr unsigned kRowsBytes = (unsigned)NR * (MB + MB + 4u);
  float v[kTmaStages][3][NP];
  MassElem<MR> m1[RS][NR], m2[RS][NR];
  float phi[RS][NR];
};
template <int TXC, int TY, int MR = kMassF64>
struct GbfPairSmem {
  using Ring = GbfPairRing<TXC, TY, MR>;
  Ring ring;
  float dP[kTmaStages][Ring::NP];
  float L1[kTmaStages][Ring::NP], L2[kTmaStages][Ring::NP];
};
// The mbarriers of the two rings (halo planes, interior rows), apart from the
// ring data: a CTA that runs tiles of two shapes keeps one set of barriers,
// and their parities, for both.
template <int MR>
struct alignas(128) GbfPairBars {
  static constexpr int RS = 3;
  unsigned long long bar[kTmaStages], mbar[RS];
};
// Dynamic shared memory of an x-pair CTA: barriers, then one shape's rings and
// plane buffers (every TMA destination on a 128-byte boundary).
template <int TXC, int TY, int MR>
struct GbfPairCta {
  GbfPairBars<MR> bars;
  GbfPairSmem<TXC, TY, MR> body;
};
// The same for a CTA that runs 32x16 and 48x10 x-pair tiles (the 48-wide
// tile covers a grid's last 48 columns where nx is 16 more than a multiple of
// 32; its halo box {56, 12} is smaller than {40, 18}).
template <int MR>
struct GbfPairCtaMixed {
  GbfPairBars<MR> bars;
  union {
    GbfPairSmem<32, 16, MR> a;
    GbfPairSmem<48, 10, MR> b;
  };
};
template <int MR>
__device__ __forceinline__ void gbf_pair_bars_init(GbfPairBars<MR>& b) {
  for (int s = 0; s < kTmaStages; s++) gbf_mbar_init(&b.bar[s], 1);
  for (int s = 0; s < GbfPairBars<MR>::RS; s++) gbf_mbar_init(&b.mbar[s], 1);
  gbf_mbar_fence_init();
}

__device__ __forceinline__ float2 gbf_ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void gbf_st2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }

// Address of cell c of a mass array (8 or 4 bytes a cell), as the array's nominal type.
template <int MR>
__device__ __forceinline__ double* mass_at(double* p, size_t c) {
  return reinterpret_cast<double*>(reinterpret_cast<MassElem<MR>*>(p) + c);
}
template <int MR> struct WidePair;
template <> struct WidePair<kMassF64> {  // FP64 masses: two doubles
  static __device__ __forceinline__ void load(const double* p, double& a, double& b) {
    const double2 v = *reinterpret_cast<const double2*>(p);
    a = v.x;
    b = v.y;
  }
  static __device__ __forceinline__ void store(double* p, double a, double b) {
    *reinterpret_cast<double2*>(p) = make_double2(a, b);
  }
};
template <> struct WidePair<kMassDF> {  // FP32-pair masses: four floats
  static __device__ __forceinline__ void load(const double* p, GbfDF& a, GbfDF& b) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    a = {v.x, v.y};
    b = {v.z, v.w};
  }
  static __device__ __forceinline__ void store(double* p, GbfDF a, GbfDF b) {
    *reinterpret_cast<float4*>(p) = make_float4(a.hi, a.lo, b.hi, b.lo);
  }
};
template <> struct WidePair<kMassDefectDF> : WidePair<kMassDF> {};  // pair defects: four floats
template <> struct WidePair<kMassDefect> {  // FP32 defects: two floats
  static __device__ __forceinline__ void load(const double* p, float& a, float& b) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    a = v.x;
    b = v.y;
  }
  static __device__ __forceinline__ void store(double* p, float a, float b) {
    *reinterpret_cast<float2*>(p) = make_float2(a, b);
  }
};

// The x-pair z-marching tile: cells x0 .. x0 + TXC - 1 (interior ones only)
// of rows j0 .. j0 + TY - 1, planes k0 .. k1 - 1. Same staging protocol,
// bounded waits and give-up as split_tile<..., TMA = true>; each cell is
// updated by split_cell, so results equal the other tiles' bit for bit. The
// CTA has NTB >= TXC / 2 * TY threads; the ones beyond the tile take part in
// the barriers only.
template <int MR, int TXC, int TY, bool CFL = false, int NTB = TXC / 2 * TY, bool PATCH = false>
__device__ bool split_tile_x2(const GbfSplitConsts& C, const GbfSplitGrid& G, int x0, int j0, int k0, int k1,
                              GbfPairBars<MR>& bars, GbfPairSmem<TXC, TY, MR>& sm, GbfSplitAcc<MR>& acc,
                              const GbfTmaSet* maps, int buf, unsigned* phases) {
  using W = WideOf<MR>;
  using WT = typename W::T;
  using MT = typename MassRep<MR>::T;
  using Ring = GbfPairRing<TXC, TY, MR>;
  constexpr int THX = TXC / 2, NT = THX * TY, BX = Ring::BX, HY = Ring::HY, RS = Ring::RS;
  static_assert(NT <= NTB && RS == GbfPairBars<MR>::RS, "x-pair CTA shape");
  constexpr int PCOLS = (TXC + 4) / 2;  // pair columns 1 .. PCOLS of the box (columns 2 .. TXC + 5)
  constexpr int NPAIR = PCOLS * HY, SLOTS = (NPAIR + NT - 1) / NT;
  Ring& raw = sm.ring;
  const bool in_tile = NT == NTB || (int)threadIdx.x < NT;
  const int nx = C.nx, ny = C.ny;
  const unsigned pln = (unsigned)nx * (unsigned)ny;
  const int tx = threadIdx.x % THX, ty = threadIdx.x / THX;
  const int ia = x0 + 2 * tx, j = j0 + ty;
  const bool row_ok = in_tile && j <= ny - 2;
  const bool act_a = row_ok && ia >= 1 && ia <= nx - 2;
  const bool act_b = row_ok && ia + 1 <= nx - 2;
  const bool any = row_ok && ia <= nx - 2;  // the pair lies in the grid's row (cell b at most nx - 1)
  const int hc = (ty + 1) * BX + 2 * tx + 4;  // own pair in the plane buffers (even)
  const int mi = ty * TXC + 2 * tx;           // own pair in the rows boxes (even)

  // halo pairs of this thread: even plane index, global row (rows or columns
  // outside the grid hold zeros and give finite, unused properties). Slot 0
  // is the thread's own pair (box row ty + 1); then the interior pairs of the
  // halo rows 0 and HY - 1, then the left and right halo pair of every row.
  // The pairs of a row go to consecutive threads (a row's THX pairs are
  // contiguous in shared memory: no bank conflicts).
  // (slot 0 is hc in row j: only the other slots keep their positions)
  int hq[SLOTS], hj[SLOTS];
#pragma unroll
  for (int s = 1; s < SLOTS; s++) {
    const int q = threadIdx.x + s * NT;
    hq[s] = -1;
    hj[s] = 0;
    if (in_tile && q < NPAIR) {
      int r, c2;
      if (q < NT + 2 * THX) {
        const int h = q - NT;
        r = h < THX ? 0 : HY - 1;
        c2 = 2 + h % THX;
      } else {
        const int h = q - NT - 2 * THX;
        r = h >> 1;
        c2 = (h & 1) ? PCOLS : 1;
      }
      hq[s] = r * BX + 2 * c2;
      hj[s] = j0 - 1 + r;
    }
  }

  // Both rings have three stages: plane p uses stage (p - k0) % 3 of each, so
  // one rotating index u = (k - k0) % 3 names every stage the loop touches.
  static_assert(RS == kTmaStages && kTmaStages == 3, "x-pair rings");
  unsigned pend = 0;
  auto issue = [&](int p, int s) {  // halo planes of plane p into stage s
    if (threadIdx.x == 0) {
      gbf_mbar_expect_tx(&bars.bar[s], Ring::kHaloBytes);
      gbf_tma_plane(raw.v[s][0], &maps->dP[buf], x0 - 4, j0 - 1, p, &bars.bar[s]);
      gbf_tma_plane(raw.v[s][1], &maps->S[buf], x0 - 4, j0 - 1, p, &bars.bar[s]);
      gbf_tma_plane(raw.v[s][2], &maps->K, x0 - 4, j0 - 1, p, &bars.bar[s]);
    }
    pend |= 1u << s;
  };
  auto issue_rows = [&](int p, int s) {  // M1, M2, phi rows of plane p into stage s
    if (threadIdx.x == 0) {
      gbf_mbar_expect_tx(&bars.mbar[s], Ring::kRowsBytes);
      gbf_tma_plane(raw.m1[s], &maps->M1, x0, j0, p, &bars.mbar[s]);
      gbf_tma_plane(raw.m2[s], &maps->M2, x0, j0, p, &bars.mbar[s]);
      gbf_tma_plane(raw.phi[s], &maps->phi, x0, j0, p, &bars.mbar[s]);
    }
    pend |= 1u << (8 + s);
  };
  auto wait_bit = [&](int bit) -> bool {
    unsigned long long* b = bit < 8 ? &bars.bar[bit] : &bars.mbar[bit - 8];
    if (!gbf_mbar_wait(b, (*phases >> bit) & 1u, kTmaWaitTries)) return false;
    *phases ^= 1u << bit;
    pend &= ~(1u << bit);
    return true;
  };
  auto give_up = [&]() {
    for (int bit = 0; bit < 16; bit++)
      if ((pend >> bit) & 1u) {
        unsigned long long* b = bit < 8 ? &bars.bar[bit] : &bars.mbar[bit - 8];
        gbf_mbar_wait(b, (*phases >> bit) & 1u, kTmaDrainTries);
        *phases ^= 1u << bit;
      }
    pend = 0;
    if (threadIdx.x == 0) atomicOr(G.status, GBF_DEV_TIMEOUT);
  };
  float2 s_own = make_float2(0.f, 0.f);  // S of the own pair in the plane built last
  auto build = [&](int s) {  // plane buffer s from halo stage s
#pragma unroll
    for (int q = 0; q < SLOTS; q++) {
      // slot 0: the own pair of every thread in the tile; the first later
      // slots hold a pair for every thread too where the halo is large enough
      if (q == 0 ? in_tile : ((NT == NTB && (q + 1) * NT <= NPAIR) || hq[q] >= 0)) {
        const int e = q == 0 ? hc : hq[q], jr = q == 0 ? j : hj[q];
        const float2 p = gbf_ld2(&raw.v[s][0][e]), sv = gbf_ld2(&raw.v[s][1][e]), kv = gbf_ld2(&raw.v[s][2][e]);
        float l1a, l2a, l1b, l2b;
        split_props(C, 0, kv.x, p.x, sv.x, jr, l1a, l2a);
        split_props(C, 0, kv.y, p.y, sv.y, jr, l1b, l2b);
        gbf_st2(&sm.dP[s][e], p.x, p.y);
        gbf_st2(&sm.L1[s][e], l1a, l1b);
        gbf_st2(&sm.L2[s][e], l2a, l2b);
        if (q == 0) s_own = sv;
      }
    }
  };

  // prologue: own pair at k0 - 1 (registers), plane k0 (shared)
  for (int q = 0; q < kTmaStages && k0 + q <= k1; q++) issue(k0 + q, q);
  for (int q = 0; q < RS && k0 + q < k1; q++) issue_rows(k0 + q, q);
  float dPma = 0.f, L1ma = 0.f, L2ma = 0.f, dPmb = 0.f, L1mb = 0.f, L2mb = 0.f;
  if (any) {
    const unsigned c = (unsigned)(ia + j * nx) + (unsigned)(k0 - 1) * pln;
    const float2 p = gbf_ld2(G.dP + c), sv = gbf_ld2(G.S + c), kv = gbf_ld2(G.K + c);
    dPma = p.x;
    dPmb = p.y;
    split_props(C, 0, kv.x, p.x, sv.x, j, L1ma, L2ma);
    split_props(C, 0, kv.y, p.y, sv.y, j, L1mb, L2mb);
  }
  {
    const bool ok = wait_bit(0);
    if (ok) build(0);
    if (__syncthreads_or(!ok)) {
      give_up();
      return false;
    }
    if (k0 + kTmaStages <= k1) issue(k0 + kTmaStages, 0);
  }
  // flux carry of both cells: the faces between planes k0 - 1 and k0
  float fza1 = 0.f, fza2 = 0.f, fzb1 = 0.f, fzb2 = 0.f;
  if (any) {
    const float2 d = gbf_ld2(sm.dP[0] + hc), a = gbf_ld2(sm.L1[0] + hc), b = gbf_ld2(sm.L2[0] + hc);
    split_zface(C, dPma, L1ma, L2ma, d.x, a.x, b.x, fza1, fza2);
    split_zface(C, dPmb, L1mb, L2mb, d.y, a.y, b.y, fzb1, fzb2);
  }
  const WT R01 = W::c(C.ro01_d, C.ro01_df), R02 = W::c(C.ro02_d, C.ro02_df);
  const GbfDefectRow rw = gbf_is_defect(MR) ? gbf_defect_row(C, j) : GbfDefectRow{};
  const int cols[2] = {ia, ia + 1};
  const unsigned rowf = split_row_flags<2>(C, j, cols);
  const bool hsides = C.noflow_bottom != 0;  // x faces: hydrostatic Dirichlet (dP = 0)
  if constexpr (gbf_is_defect(MR)) {
    acc.c1 = rw.c1;
    acc.c2 = rw.c2;
  }
  int u = 0;  // (k - k0) % 3: plane buffer, halo stage and rows stage of plane k
  for (int k = k0; k < k1; k++) {
    const float2 s0 = s_own;  // plane k's, before the build of plane k + 1 replaces it
    const int t_cur = u, t_next = u == 2 ? 0 : u + 1, t_rows = u;
    {
      const int sn = t_next;
      bool ok = wait_bit(sn);
      ok = ok && wait_bit(8 + t_rows);
      if (ok) build(sn);
      if (__syncthreads_or(!ok)) {
        give_up();
        return false;
      }
      // halo stage sn was consumed by the build above; rows stage (u + 2) % 3
      // (plane k - 1) by the previous plane's update
      if (k + 1 + kTmaStages <= k1) issue(k + 1 + kTmaStages, sn);
      if (k > k0 && k + 2 < k1) issue_rows(k + 2, sn == 2 ? 0 : sn + 1);
    }
    if (any) {
      const float* Pd = sm.dP[t_cur];
      const float* P1 = sm.L1[t_cur];
      const float* P2 = sm.L2[t_cur];
      const float2 d0 = gbf_ld2(Pd + hc), dl = gbf_ld2(Pd + hc - 2), dr = gbf_ld2(Pd + hc + 2);
      const float2 du = gbf_ld2(Pd + hc - BX), dd = gbf_ld2(Pd + hc + BX);
      const float2 a0 = gbf_ld2(P1 + hc), al = gbf_ld2(P1 + hc - 2), ar = gbf_ld2(P1 + hc + 2);
      const float2 au = gbf_ld2(P1 + hc - BX), ad = gbf_ld2(P1 + hc + BX);
      const float2 b0 = gbf_ld2(P2 + hc), bl = gbf_ld2(P2 + hc - 2), br = gbf_ld2(P2 + hc + 2);
      const float2 bu = gbf_ld2(P2 + hc - BX), bd = gbf_ld2(P2 + hc + BX);
      const float2 dp = gbf_ld2(sm.dP[t_next] + hc), ap = gbf_ld2(sm.L1[t_next] + hc),
                   bp = gbf_ld2(sm.L2[t_next] + hc);
      const float2 ph = gbf_ld2(&raw.phi[t_rows][mi]);
      MT M1a, M1b, M2a, M2b;
      WidePair<MR>::load(reinterpret_cast<const double*>(&raw.m1[t_rows][mi]), M1a, M1b);
      WidePair<MR>::load(reinterpret_cast<const double*>(&raw.m2[t_rows][mi]), M2a, M2b);
      GbfCellIn in[2];
      // cell a
      in[0].dPc = d0.x; in[0].S0 = s0.x; in[0].L1c = a0.x; in[0].L2c = b0.x;
      in[0].dPxm = dl.y; in[0].dPxp = d0.y; in[0].dPym = du.x; in[0].dPyp = dd.x;
      in[0].L1xm = al.y; in[0].L1xp = a0.y; in[0].L1ym = au.x; in[0].L1yp = ad.x;
      in[0].L2xm = bl.y; in[0].L2xp = b0.y; in[0].L2ym = bu.x; in[0].L2yp = bd.x;
      in[0].fz1 = fza1; in[0].fz2 = fza2;
      in[0].dPp = dp.x; in[0].L1p = ap.x; in[0].L2p = bp.x;
      in[0].phi = ph.x;
      // cell b
      in[1].dPc = d0.y; in[1].S0 = s0.y; in[1].L1c = a0.y; in[1].L2c = b0.y;
      in[1].dPxm = d0.x; in[1].dPxp = dr.x; in[1].dPym = du.y; in[1].dPyp = dd.y;
      in[1].L1xm = a0.x; in[1].L1xp = ar.x; in[1].L1ym = au.y; in[1].L1yp = ad.y;
      in[1].L2xm = b0.x; in[1].L2xp = br.x; in[1].L2ym = bu.y; in[1].L2yp = bd.y;
      in[1].fz1 = fzb1; in[1].fz2 = fzb2;
      in[1].dPp = dp.y; in[1].L1p = ap.y; in[1].L2p = bp.y;
      in[1].phi = ph.y;
      const MT m1s[2] = {M1a, M1b}, m2s[2] = {M2a, M2b};
      const bool cnt[2] = {act_a, act_b};
      GbfCellOut<MR> o[2];
      split_cells<MR, 2, CFL, PATCH>(C, in, m1s, m2s, R01, R02, rw, 0, rowf, j, k, true, G.mass_partials != nullptr,
                                     cnt, acc, o, G.patch_in, ia);
      // The x faces i = 0 and i = nx - 1 (rows and planes interior) take the
      // boundary rules' values here: the new S of the x-neighbour and its dP
      // (cpu.cpp:327-331, 366-372), or the hydrostatic side value dP = 0 with
      // GBF_BC_HYDROSTATIC_SIDES; no other boundary rule reads these cells, so
      // the face pass skips them (gbf_boundary_count_no_xfaces, gbf_face_row).
      const GbfCellOut<MR> oa = act_a ? o[0] : GbfCellOut<MR>{hsides ? 0.f : o[1].dPn, o[1].Sn, M1a, M2a};
      const GbfCellOut<MR> ob = act_b ? o[1] : GbfCellOut<MR>{hsides ? 0.f : o[0].dPn, o[0].Sn, M1b, M2b};
      const unsigned c = (unsigned)(ia + j * nx) + (unsigned)k * pln;  // even: nx and ia are
      gbf_st2(G.dPn + c, oa.dPn, ob.dPn);
      gbf_st2(G.Sn + c, oa.Sn, ob.Sn);
      WidePair<MR>::store(mass_at<MR>(G.M1, c), oa.M1n, ob.M1n);
      WidePair<MR>::store(mass_at<MR>(G.M2, c), oa.M2n, ob.M2n);
      fza1 = o[0].fz1; fza2 = o[0].fz2;
      fzb1 = o[1].fz1; fzb2 = o[1].fz2;
    }
    u = t_next;
  }
  return true;
}

// ------------------------------------------------ the Dirichlet patch's inflow
// The DNAPL mass per pore volume that the j = 1 cell c gains this step through
// its face with the patch cell c - nx above it, in FP64 from the stored FP32
// state: the face potential with the centre cell's density (cpu.cpp:257-258)
// and the donor-cell product (cpu.cpp:260-262), the patch cell's mobility at
// exactly S2_gr (the boundary rules, cpu.cpp:343-362). dPb, dPc: the stored
// pressure deviations of the patch cell and of c; Sc the stored S of c.
__device__ __forceinline__ double split_patch_inflow(const GbfSplitConsts& C, const GbfPatchConsts& P,
                                                     const GbfSplitGrid& G, unsigned c, int md, int mdb, float dPb,
                                                     float dPc, float Sc, double phi) {
  const unsigned b = c - (unsigned)C.nx;
  const double Ppc = C.H_d + (double)dPc;                   // P - P_atm at the cell (j = 1)
  const double rho2c = C.ro02_d * (1.0 + C.beta2_d * Ppc);  // the centre cell's density
  const double pot = ((double)dPb - (double)dPc) - C.H_d + rho2c * P.gh2;  // h2 times the potential
  auto mobility = [&](double K, int mdx, double S, double Pp) {
    const double Se = 1.0 + S * P.se_b[mdx];
    const double kr2 = (1.0 - Se) * (1.0 - Se) * (1.0 - pow(Se, P.e2[mdx]));
    return K * kr2 * P.nmr2 * (1.0 + C.beta2_d * Pp);
  };
  const double L = pot >= 0.0 ? mobility(G.K ? (double)G.K[b] : P.K[mdb], mdb, P.S2, (double)dPb)
                              : mobility(G.K ? (double)G.K[c] : P.K[md], md, (double)Sc, Ppc);
  return -(pot * L) * P.wy / phi;
}

// The pre-pass of a step under the Dirichlet patch, patch cell t of n x n
// (i = i0 + t % n, k = k0 + t / n), on the state the step starts from: the
// j = 1 cell's FP64 DNAPL inflow into G.patch_in[t], as an FP32 pair, which
// the step's tiles (PATCH) take in place of that face's FP32 flux. Where DNAPL
// enters through the patch, every kilogram of it crosses these faces, so FP32
// mobilities there (the hardware log2 / exp2, about 2^-22) would set the
// relative precision of the whole DNAPL total. Cells of the patch's columns
// outside the grid's interior are skipped (no tile reads them).
__device__ __forceinline__ void gbf_split_patch_cell(const GbfSplitConsts& C, const GbfPatchConsts& P,
                                                     const GbfSplitGrid& G, int t) {
  const int i = P.i0 + t % P.n, k = P.k0 + t / P.n;
  if (i < 1 || i > C.nx - 2 || k < 1 || k > C.nz - 2 || C.ny < 3) return;
  const unsigned c = (unsigned)(i + C.nx) + (unsigned)k * (unsigned)C.nx * (unsigned)C.ny;  // j = 1
  const unsigned b = c - (unsigned)C.nx;                                                     // the patch cell
  const int md = G.media ? G.media[c] : 0, mdb = G.media ? G.media[b] : 0;
  const double phi = G.phi ? (double)G.phi[c] : C.m_d[md];
  G.patch_in[t] = gbf_df_from_double(split_patch_inflow(C, P, G, c, md, mdb, G.dP[b], G.dP[c], G.S[c], phi));
}
