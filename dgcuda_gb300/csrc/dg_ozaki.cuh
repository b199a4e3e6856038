// dg_ozaki.cuh -- the element kernel's basis contractions on the tensor
// cores with FP64 accuracy (exact-slice emulation after Ozaki, Ogita and
// Oishi, "Error-free transformations of matrix multiplication by using fast
// routines of matrix multiplication and its applications", Numer. Algorithms
// 59, 2012; slices held as small integers, as in Ootomo, Ozaki and Yokota,
// IJHPCA 2024).
//
// GB300 runs FP64 FMAs at 2 per SM per cycle and f16 tensor MMAs at ~960
// multiply-adds per SM per cycle (mma.sync, measured), so the element kernel
// is bound by its FP64 basis contractions: u(q) = sum_i c_i phi_i(q) at the
// area points, the projection sum_q (GR_qi g_q + GS_qi h_q), the surface
// gather sum_fj E_fji F_fj and the next stage's edge traces.  Here each of
// them runs as exact integer arithmetic on the tensor cores:
//
//  * a row of inputs (one element and variable) shares the exponent of its
//    largest entry; each entry becomes a 53-bit integer X (truncated), and X
//    is written in 7 balanced base-256 digits d_j in [-128, 127]
//    (X + 0x80808080808080 has the unsigned digits d_j + 128);
//  * the table columns are split the same way (on the host);
//  * every digit pair (i, j) with i + j >= 5 is one f16 MMA with f32
//    accumulation; pairs of equal weight 256^(i+j) share an accumulator.  A
//    product is at most 2^14, a weight class has at most 7 pairs, a group
//    accumulates at most 36 real K slots, so every partial sum is an
//    integer below 7 * 36 * 2^14 < 2^22 in magnitude: the accumulator starts at 1.5 * 2^23, where
//    fp32 holds every integer of the window exactly, and the integer is read
//    back from its bits;
//  * the 8 weight sums are combined into one 128-bit integer and rounded
//    to the nearest double with integer instructions (no FP64 work).
//  The pairs left out (i + j < 5) and the truncation of the inputs bound the
//  error of each output by about 2^-52 max|x| max|t| times the slot count,
//  the order of an FP64 dot product's own rounding.
//
// Layout: one warp contracts 16 elements (rows g and g + 8 of the MMA, g =
// lane / 4); the 4 lanes of a quad hold K slots {2t, 2t+1, 2t+8, 2t+9} (t =
// lane % 4) of both rows, which are the positions 0..3 of the thread.  The
// D fragment of an MMA gives the thread the output columns at the same
// positions, so the four contractions chain without moving data: the area
// points the first one produces are the K slots of the projection, and the
// modes the projection produces are the K slots of the trace contraction.
// Items (modes, area points, edge points) fill the positions in the order
// position 0 of t = 0..3, position 1 of t = 0..3, and so on, so every lane
// has the same number of real items up to the last position.
#pragma once
#include <cstdint>

#include <cuda_fp16.h>

#include "dg_kernels.cuh"

namespace dg {
namespace oz {

constexpr int kDigits = 7;
constexpr int kMinPair = 5;                 // digit pairs with i + j >= 5
constexpr int kWeights = 8;                 // weight classes 12 - (i + j) = 0..7
constexpr unsigned long long kBias = 0x80808080808080ull;
constexpr float kAccInit = 12582912.0f;     // 1.5 * 2^23
constexpr int kAccBits = 0x4B400000;        // its bit pattern

// tables: EVAL (K = modes, N = area points), PROJ (3 K blocks: GR and GS
// over the area points, E over the edge points; N = modes; one exponent per
// column across the three), TRACE (K = modes, N = edge points).  Words are
// the B fragments of each lane: word[digit][kblock][colgroup][lane] =
// {k 2t..2t+1, k 2t+8..2t+9} of column colgroup * 8 + g, as f16 pairs.
enum { kEval = 0, kProj = 1, kTrace = 2 };
// word offset of each table: 7 digits x 2 column groups x 32 lanes per K
// block, K blocks 1, 3, 1
__host__ __device__ constexpr int word_off(int tab) { return 7 * 2 * 32 * (tab == 0 ? 0 : tab == 1 ? 1 : 4); }
constexpr int kWords = 7 * 5 * 2 * 32;      // 2240 uint2
struct Tabs {
  uint2 w[kWords];
  int colexp[3][16];                         // biased exponent of each table column
  int pad[16];
};

// position p of lane quad index t -> slot (0..15); item index of (p, t)
__host__ __device__ constexpr int slot_of(int pos, int t) { return pos < 2 ? 2 * t + pos : 2 * t + 8 + (pos - 2); }
__host__ __device__ constexpr int npos(int items) { return (items + 3) / 4; }

// ---- per-value splitting --------------------------------------------------
__device__ __forceinline__ int bexp(double x) {
  return (__double2hiint(x) >> 20) & 0x7FF;
}

// 53-bit fixed point of x on a row whose largest biased exponent is m, plus
// the digit bias (see above)
__device__ __forceinline__ long long to_fixed(double x, int m) {
  const long long b = __double_as_longlong(x);
  const int eb = (int)((b >> 52) & 0x7FF);
  const unsigned long long mant =
      ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | (eb ? (1ull << 52) : 0ull);
  const int sh = m - (eb ? eb : 1);
  unsigned long long X = sh < 64 ? (mant >> sh) : 0ull;
  long long v = b < 0 ? -(long long)X : (long long)X;
  return v + (long long)kBias;
}

// f16 pair of digit j of two biased fixed-point values (low half: a)
template <int J>
__device__ __forceinline__ uint32_t digit_pair(long long a, long long b) {
  const uint32_t wa = J < 4 ? (uint32_t)a : (uint32_t)((unsigned long long)a >> 32);
  const uint32_t wb = J < 4 ? (uint32_t)b : (uint32_t)((unsigned long long)b >> 32);
  constexpr uint32_t s = (J % 4) | ((4 + (J % 4)) << 8);
  const uint32_t u = (__byte_perm(wa, wb, s) & 0x00FF00FFu) | 0x64006400u;  // 1024 + u
  __half2 h = *reinterpret_cast<const __half2 *>(&u);
  h = __hsub2(h, __halves2half2(__ushort_as_half(0x6480), __ushort_as_half(0x6480)));  // - 1152
  return *reinterpret_cast<const uint32_t *>(&h);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// the same for a K block that uses only K slots 0..7 (thread positions 0 and
// 1): the first halves of the k16 fragments
__device__ __forceinline__ void mma1688(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t b) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(b));
}

// accumulators of one output group: [weight][colgroup][fragment]
struct Acc {
  float d[kWeights][2][4];
  __device__ __forceinline__ void reset() {
#pragma unroll
    for (int w = 0; w < kWeights; w++)
#pragma unroll
      for (int c = 0; c < 2; c++)
#pragma unroll
        for (int r = 0; r < 4; r++) d[w][c][r] = kAccInit;
  }
};

// one K block: Y[e][pos] are the biased fixed-point inputs of rows e = 0
// (g) and 1 (g + 8) at the thread's positions; W points at the block's
// words in global memory (digit stride 2 * KB * 32; the 18 KB of words stay
// in L1)
// (NCG: how many of the two column groups of 8 outputs are needed; K8: the
// block's inputs fill only positions 0 and 1.  At p <= 2 the area points and
// modes fill only the first column group and K slots 0..7)
template <int KB, int NCG = 2, bool K8 = false>
__device__ __forceinline__ void contract(Acc &acc, const long long (&Y)[2][4], const uint2 *W,
                                         int kb, int lane) {
  uint32_t A[kDigits][4];
#define DG_OZ_DIG(J)                                 \
  A[J][0] = digit_pair<J>(Y[0][0], Y[0][1]);         \
  A[J][1] = digit_pair<J>(Y[1][0], Y[1][1]);         \
  A[J][2] = digit_pair<J>(Y[0][2], Y[0][3]);         \
  A[J][3] = digit_pair<J>(Y[1][2], Y[1][3]);
  DG_OZ_DIG(0) DG_OZ_DIG(1) DG_OZ_DIG(2) DG_OZ_DIG(3) DG_OZ_DIG(4) DG_OZ_DIG(5) DG_OZ_DIG(6)
#undef DG_OZ_DIG
#pragma unroll
  for (int i = 0; i < kDigits; i++) {
    const uint2 b0 = __ldg(&W[((i * KB + kb) * 2 + 0) * 32 + lane]);
    const uint2 b1 = NCG > 1 ? __ldg(&W[((i * KB + kb) * 2 + 1) * 32 + lane]) : b0;
#pragma unroll
    for (int j = 0; j < kDigits; j++) {
      if (i + j < kMinPair) continue;
      const int w = 2 * (kDigits - 1) - i - j;
      if (K8) {
        mma1688(acc.d[w][0], A[j][0], A[j][1], b0.x);
        if (NCG > 1) mma1688(acc.d[w][1], A[j][0], A[j][1], b1.x);
      } else {
        mma16816(acc.d[w][0], A[j], b0);
        if (NCG > 1) mma16816(acc.d[w][1], A[j], b1);
      }
    }
  }
}

// output at fragment entry (cg, r): row exponent m (biased, of the row of
// r >> 1), column exponent M (biased).  The value is S 2^k with the exact
// integer S = sum_w d_w 256^(7 - w) (below 2^79 in magnitude) and k = m + M
// - 2110; it is rounded to the nearest double (ties to even) with integer
// instructions only: S as a 128-bit two's complement pair, its magnitude
// normalised by a leading-zero count, 53 bits kept, the rest as round and
// sticky bits.
static __device__ __noinline__ double recombine_sums(int d0, int d1, int d2, int d3, int d4, int d5,
                                             int d6, int d7, int m, int M) {
  const int d[kWeights] = {d0, d1, d2, d3, d4, d5, d6, d7};
  const long long Sh = (long long)d[0] * 65536 + (long long)d[1] * 256 + d[2];  // |Sh| < 2^39
  const long long Sl = (long long)d[3] * 4294967296ll + (long long)d[4] * 16777216 +
                       (long long)d[5] * 65536 + (long long)d[6] * 256 + d[7];  // |Sl| < 2^55
  // S = Sh 2^40 + Sl as (hi, lo)
  unsigned long long lo = (unsigned long long)Sh << 40;
  long long hi = Sh >> 24;
  const unsigned long long l2 = lo + (unsigned long long)Sl;
  hi += (Sl >> 63) + (l2 < lo ? 1 : 0);
  lo = l2;
  const bool neg = hi < 0;
  if (neg) {
    lo = ~lo + 1;
    hi = ~hi + (lo == 0 ? 1 : 0);
  }
  if (hi == 0 && lo == 0) return 0.0;
  const unsigned long long uh = (unsigned long long)hi;
  int lz;
  unsigned long long top, rest;
  if (uh) {
    lz = __clzll(uh);
    top = lz ? (uh << lz) | (lo >> (64 - lz)) : uh;
    rest = lz ? lo << lz : lo;
  } else {
    lz = 64 + __clzll(lo);
    top = lo << (lz - 64);
    rest = 0;
  }
  unsigned long long mant = top >> 11;  // 53 bits; its unit is 2^(75 - lz) in S
  const unsigned long long rbit = (top >> 10) & 1, sticky = ((top & 0x3FF) | rest) != 0;
  mant += rbit & (sticky | (mant & 1));
  int ex = 75 - lz;
  if (mant >> 53) {
    mant >>= 1;
    ex++;
  }
  const int k = m + M - 2110, e = ex + 52 + k + 1023;
  if (e >= 1 && e <= 2046)
    return __longlong_as_double((long long)((neg ? 1ull << 63 : 0ull) | ((unsigned long long)e << 52) |
                                            (mant & 0xFFFFFFFFFFFFFull)));
  // out of the normal range: scale in two steps (never on physical data)
  const double v = ldexp((double)(long long)mant, ex);
  return ldexp(neg ? -v : v, k);
}

// one copy of the recombination for every call site (the kernel's hot loop
// then fits the instruction cache); the class sums leave the accumulator in
// registers
__device__ __forceinline__ double recombine(const Acc &acc, int cg, int r, int m, int M) {
  if (m == 0) return 0.0;  // an all-zero (or denormal-only) row
  int d[kWeights];
#pragma unroll
  for (int w = 0; w < kWeights; w++) d[w] = __float_as_int(acc.d[w][cg][r]) - kAccBits;
  return recombine_sums(d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], m, M);
}

// a hint that the line holding p will be read soon (no register is held)
__device__ __forceinline__ void prefetch_l1(const void *p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// largest biased exponent over a quad's row (all 4 lanes hold the result)
__device__ __forceinline__ int quad_max(int m) {
  m = max(m, __shfl_xor_sync(0xffffffffu, m, 1));
  return max(m, __shfl_xor_sync(0xffffffffu, m, 2));
}


// ---------------------------------------------------------------------------
// The fused SSP-RK3 element stage (element_body<Eq, P, true>) with the four
// basis contractions on the tensor cores.  Same inputs, outputs and rules as
// element_body: volume integral (flattened to the element mean if an area
// point is non-physical), surface gather (-F on a left face, +F at the
// mirrored points on a right face), 1/J, the RK combination, the next
// stage's edge traces and their positivity check.  A block is 4 warps of 16
// elements; equations without a bed source.  The loops over variables are
// not unrolled (one copy of each contraction in the code); what crosses
// them -- area values, metric-folded fluxes, new traces -- is staged per
// warp in shared memory, each lane in its own column.
constexpr int kOzThreads = 128, kOzElems = 64;  // k_trace_oz: 4 warps of 16 elements

// the element stage's block: warps (of 16 elements) per block and blocks per
// SM, from its shared memory (GH doubles per lane) and registers.  5 warps
// on an SM sub-partition leave 96 registers a thread (102 rounded down):
// p = 2 runs 5 blocks of 4 warps there (32 KB of staging per block, 5 %
// faster than 4 blocks at 128); p = 3 keeps 4 blocks at 128 (48 KB per
// block; 6 blocks of 3 warps at 96 registers measured 26 % slower) and
// p = 4 3 blocks at 168 (64 KB; 7 blocks of 2 warps at 128, 19 % slower).
template <int P> struct OzBlock {
  static constexpr int kWarps = 4;
  static constexpr int kPerSM = P == 2 ? 5 : P == 4 ? 3 : 4;
  static constexpr int kThreads = 32 * kWarps, kElems = 16 * kWarps;
};

template <class Eq, int P>
struct OzShape {
  static constexpr int N = Eq::N, NP = Tab<P>::NP, NQ = Tab<P>::NQ, N1 = Tab<P>::N1, NF = 3 * N1;
  static constexpr int PM = npos(NP), PQ = npos(NQ), PF = npos(NF);
  // g, h per (position, row, variable) and lane; the area values and the
  // new traces live in the same slots (gh_slot)
  static constexpr int GH = 2 * PQ * 2 * N;
  static_assert(PF <= 2 * PQ, "the traces of a variable fit its g, h slots");
  // a variable's g/h position PF, unused by its traces: where the fused
  // limiter keeps modes 1 and 2 of the unlimited output (p >= 2)
  static constexpr bool kStash = PF < 2 * PQ;
  static constexpr size_t kSmem = (size_t)OzBlock<P>::kWarps * GH * 32 * sizeof(double);
};

// per-warp staging, one column per lane: slot k (0: g, 1: h) of variable n
// at position p of row e.  An area value u(n, p, e) sits in the g slot of
// its own (p, e), which the flux phase reads before writing g and h there;
// the new trace at position p' of variable n goes to slot (p' / 2, e,
// p' % 2) of that variable, whose g and h the projection has already read
template <int N>
__device__ __forceinline__ int gh_slot(int n, int p, int e, int k) {
  return (((p * 2 + e) * N + n) * 2 + k) * 32;
}

template <class Eq, int P>
constexpr size_t oz_smem_bytes() { return OzShape<Eq, P>::kSmem; }

// row exponents (quad-reduced) and biased fixed-point values of two rows
__device__ __forceinline__ void split_rows(const double (&x)[2][4], int (&m)[2],
                                           long long (&Y)[2][4]) {
#pragma unroll
  for (int e = 0; e < 2; e++) {
    int mm = 0;
#pragma unroll
    for (int p = 0; p < 4; p++) mm = max(mm, bexp(x[e][p]));
    m[e] = quad_max(mm);
#pragma unroll
    for (int p = 0; p < 4; p++) Y[e][p] = to_fixed(x[e][p], max(m[e], 1));
  }
}

// The limiter in the element stage's epilogue (limit_tr_body's rules), after
// the stage has written its unlimited output and staged its new traces in gh.
// Lane t of a quad limits variable t of the quad's two elements, so alpha and
// the bounds are found once per element and variable (N <= 4):
//  * each lane takes the extremes of the staged traces at its own positions,
//    for every variable, as order keys on the integer pipe; a reduce-scatter
//    over the quad leaves lane t the extremes of variable t;
//  * lane t forms the bounds from the means of the element and its three
//    neighbours (a.M, a.nbr) and alpha;
//  * where alpha < 1 it scales modes 1 and 2 (from the stash slot, else from
//    the output) in the output, drops the higher modes and rebuilds all of
//    variable t's staged traces (every position, in the four lanes'
//    columns): the mean where alpha = 0, else a0 + c1 E_1 + c2 E_2, with
//    compile-time table indices.
template <class Eq, int P>
__device__ __forceinline__ void limit_epilogue(const Tab<P> &tab, const ElemArgs &a, double *gh,
                                               int lane, const int (&ec)[2], const int (&el)[2],
                                               const bool (&live)[2]) {
  using S = OzShape<Eq, P>;
  constexpr int N = S::N, NP = S::NP, N1 = S::N1, NF = S::NF, PF = S::PF;
  static_assert(N <= 4, "one variable per lane of a quad");
  const int t = lane & 3, q0 = lane & ~3;
  const size_t Kp = a.Kp;
  const double phi0 = tab.B[0][0], e0 = tab.E[0][0][0];
  // the means of this lane's variable in both elements and their neighbours,
  // loaded first so that their latency passes under the extremes below
  const double *Mn = a.M + (size_t)(t < N ? t : 0) * Kp;
  double cm[2], nm[2][3];
#pragma unroll
  for (int e = 0; e < 2; e++) {
    cm[e] = Mn[ec[e]];
#pragma unroll
    for (int f = 0; f < 3; f++) nm[e][f] = Mn[a.nbr[(size_t)f * Kp + ec[e]]];
  }
  // ---- extremes: per lane and variable, then reduce-scatter over the quad
  long long kx[2][4], kn[2][4];
#pragma unroll
  for (int e = 0; e < 2; e++)
#pragma unroll
    for (int n = 0; n < 4; n++) {
      kx[e][n] = (long long)0x8000000000000000ull;
      kn[e][n] = 0x7FFFFFFFFFFFFFFFll;
      if (n >= N) continue;
#pragma unroll
      for (int p = 0; p < PF; p++)
        if (p * 4 + t < NF) {
          const long long k = order_key(gh[gh_slot<N>(n, p >> 1, e, p & 1) + lane]);
          kx[e][n] = max(kx[e][n], k);
          kn[e][n] = min(kn[e][n], k);
        }
    }
  // step 1 (partner t ^ 1): keep the variables whose bit 0 is t's, send the
  // others; step 2 (partner t ^ 2): the same on bit 1 -- lane t ends with t
  const bool b0 = t & 1, b1 = t & 2;
  long long hx[2][2], hn[2][2];
#pragma unroll
  for (int e = 0; e < 2; e++)
#pragma unroll
    for (int h = 0; h < 2; h++) {  // variables 2h + {0, 1}
      const long long sx = b0 ? kx[e][2 * h] : kx[e][2 * h + 1];
      const long long sn = b0 ? kn[e][2 * h] : kn[e][2 * h + 1];
      const long long rx = __shfl_xor_sync(0xffffffffu, sx, 1);
      const long long rn = __shfl_xor_sync(0xffffffffu, sn, 1);
      hx[e][h] = max(b0 ? kx[e][2 * h + 1] : kx[e][2 * h], rx);
      hn[e][h] = min(b0 ? kn[e][2 * h + 1] : kn[e][2 * h], rn);
    }
  long long mx[2], mn[2];
#pragma unroll
  for (int e = 0; e < 2; e++) {
    const long long sx = b1 ? hx[e][0] : hx[e][1];
    const long long sn = b1 ? hn[e][0] : hn[e][1];
    const long long rx = __shfl_xor_sync(0xffffffffu, sx, 2);
    const long long rn = __shfl_xor_sync(0xffffffffu, sn, 2);
    mx[e] = max(b1 ? hx[e][1] : hx[e][0], rx);
    mn[e] = min(b1 ? hn[e][1] : hn[e][0], rn);
  }
  if (t >= N) return;  // (no lane is idle at N = 4)
  const int n = t;
  double *outn = a.out + (size_t)(n * NP) * Kp;
#pragma unroll
  for (int e = 0; e < 2; e++) {
    const double c0 = cm[e];
    // products reused as addends are rounded explicitly, as in limit_tr_body
    const double Uc = __dmul_rn(c0, phi0);
    double Umin, Umax;
    mean_bounds(c0, nm[e][0], nm[e][1], nm[e][2], phi0, Umin, Umax);
    const double up = fmax(0.0, from_order_key(mx[e]) - Uc);
    const double dn = fmax(0.0, Uc - from_order_key(mn[e]));
    double al = 1.0;
    const double lo = Uc - Umin, hi = Umax - Uc;
    if (up > lo) al = fmin(al, __double_as_longlong(lo) ? lo / up : 0.0);
    if (dn > hi) al = fmin(al, __double_as_longlong(hi) ? hi / dn : 0.0);
    if (al < 0.0) al = 0.0;
    if (!(al < 1.0) || !live[e]) continue;
    double c1, c2;
    if constexpr (S::kStash) {
      c1 = gh[gh_slot<N>(n, PF >> 1, e, PF & 1) + (q0 | 1)] * al;
      c2 = gh[gh_slot<N>(n, PF >> 1, e, PF & 1) + (q0 | 2)] * al;
    } else {
      c1 = outn[(size_t)1 * Kp + el[e]] * al;
      c2 = outn[(size_t)2 * Kp + el[e]] * al;
    }
    outn[(size_t)1 * Kp + el[e]] = c1;
    outn[(size_t)2 * Kp + el[e]] = c2;
#pragma unroll
    for (int i = 3; i < NP; i++) outn[(size_t)i * Kp + el[e]] = 0.0;
    // basis function 0 is constant: c0 phi_0 is one product for every point
    const double a0 = c0 * e0;
    const bool flat = al == 0.0 && a0 != 0.0;
#pragma unroll
    for (int idx = 0; idx < NF; idx++) {
      const int f = idx / N1, j = idx % N1, pp = idx >> 2, tt = idx & 3;
      double v = a0;
      if (!flat) {
        v = fma(c1, tab.E[f][j][1], v);
        v = fma(c2, tab.E[f][j][2], v);
      }
      gh[gh_slot<N>(n, pp >> 1, e, pp & 1) + (q0 | tt)] = v;
    }
  }
}

// Blocks per SM (OzBlock): 5 at p = 2, where the extra warps hide more
// latency than the spills at 96 registers cost (6 blocks at 80 registers
// slower), 4 at p = 1 and 3, 3 at p = 4.
// LIM: the limiter in the epilogue (the fused SSP-RK3 stage with the limiter
// on): the output's means are a.M (k_means, from the same stage's side-flux
// sums); each variable's new traces give its edge extremes, the means of the
// element and its three neighbours (a.nbr) give the bounds, and the limited
// modes and traces -- limit_tr_body's rules -- are what is written; the
// positivity rule is then applied to the limited traces (limit_epilogue).
template <class Eq, int P, bool LIM = false>
__global__ void __launch_bounds__(OzBlock<P>::kThreads, OzBlock<P>::kPerSM) k_element_oz(const __grid_constant__ Tab<P> tab,
                                                           const __grid_constant__ EqP q,
                                                           const __grid_constant__ ElemArgs a,
                                                           const Tabs *__restrict__ ozt) {
  static_assert(!Eq::kBathymetry, "bed source not provided on this path");
  using S = OzShape<Eq, P>;
  constexpr int N = S::N, NP = S::NP, NQ = S::NQ, N1 = S::N1, NF = S::NF;
  constexpr int PM = S::PM, PQ = S::PQ, PF = S::PF;
  static_assert(NP <= 16 && NQ <= 16 && NF <= 16, "p <= 4");
  extern __shared__ __align__(16) double smem_d[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, t = lane & 3;
  double *gh = smem_d + (size_t)warp * S::GH * 32;
  const int K = a.K, Kp = a.Kp;
  const int e0 = (blockIdx.x * OzBlock<P>::kWarps + warp) * 16 + (lane >> 2);
  const int el[2] = {e0, e0 + 8};
  const bool live[2] = {el[0] < K, el[1] < K};
  const int ec[2] = {live[0] ? el[0] : K - 1, live[1] ? el[1] : K - 1};  // loads stay in bounds
  const double *us = a.us;
  const uint2 *W = ozt->w;
  Acc acc;

  // geometry and side indices, read after the first contractions (the
  // prefetches pay from p = 3 on; at p <= 2 they cost more than they save)
  constexpr bool kPrefetch = P >= 3;
#pragma unroll
  for (int e = 0; e < 2 && kPrefetch; e++) {
#pragma unroll
    for (int r = 0; r < 5; r++) prefetch_l1(a.geo + (size_t)r * Kp + ec[e]);
#pragma unroll
    for (int f = 0; f < 3; f++) prefetch_l1(a.esd + (size_t)f * Kp + ec[e]);
  }
  // LIM: the limiter's neighbour indices and this lane's variable's mean
#pragma unroll
  for (int e = 0; e < 2 && LIM; e++) {
#pragma unroll
    for (int f = 0; f < 3; f++) prefetch_l1(a.nbr + (size_t)f * Kp + ec[e]);
    if (t < N) prefetch_l1(a.M + (size_t)t * Kp + ec[e]);
  }
  // ---- area-point values of every variable -> ub ----
#pragma unroll 1
  for (int n = 0; n < N; n++) {
    if (kPrefetch && n + 1 < N) {  // the next variable's coefficients
#pragma unroll
      for (int e = 0; e < 2; e++)
#pragma unroll
        for (int p = 0; p < PM; p++)
          if (p * 4 + t < NP) prefetch_l1(us + (size_t)((n + 1) * NP + p * 4 + t) * Kp + ec[e]);
    }
    double x[2][4];
#pragma unroll
    for (int e = 0; e < 2; e++)
#pragma unroll
      for (int p = 0; p < 4; p++) {
        const int idx = p * 4 + t;
        x[e][p] = (p < PM && idx < NP) ? us[(size_t)(n * NP + idx) * Kp + ec[e]] : 0.0;
      }
    int m[2];
    long long Y[2][4];
    split_rows(x, m, Y);
    acc.reset();
    contract<1, (PQ + 1) / 2, (PM <= 2)>(acc, Y, W + word_off(kEval), 0, lane);
#pragma unroll
    for (int p = 0; p < PQ; p++)
#pragma unroll
      for (int e = 0; e < 2; e++)
        gh[gh_slot<N>(n, p, e, 0) + lane] =
            recombine(acc, p >> 1, 2 * e + (p & 1), m[e], ozt->colexp[kEval][slot_of(p, t)]);
  }

  // ---- positivity of the area values; flatten to the element mean ----
  bool badv[2] = {false, false};
#pragma unroll
  for (int p = 0; p < PQ; p++)
#pragma unroll
    for (int e = 0; e < 2; e++) {
      if (p * 4 + t >= NQ) continue;
      double u[N];
#pragma unroll
      for (int n = 0; n < N; n++) u[n] = gh[gh_slot<N>(n, p, e, 0) + lane];
      badv[e] |= !Eq::physical(q, u);
    }
#pragma unroll
  for (int e = 0; e < 2; e++) {
    int b = badv[e];
    b |= __shfl_xor_sync(0xffffffffu, b, 1);
    b |= __shfl_xor_sync(0xffffffffu, b, 2);
    badv[e] = b != 0;
    if (badv[e]) {
#pragma unroll
      for (int n = 0; n < N; n++) {
        const double c0 = us[(size_t)(n * NP) * Kp + ec[e]];
#pragma unroll
        for (int p = 0; p < PQ; p++) {
          const int idx = p * 4 + t;
          gh[gh_slot<N>(n, p, e, 0) + lane] = c0 * tab.B[idx < NQ ? idx : 0][0];
        }
      }
    }
  }

  // ---- side-flux offsets and signs of the element's edge points ----
  int foff[PF][2];
  long long fsg[PF][2];  // sign bit of the side flux on this face (-F left, +F right)
#pragma unroll
  for (int p = 0; p < PF; p++)
#pragma unroll
    for (int e = 0; e < 2; e++) {
      const int idx = p * 4 + t;
      if (idx < NF) {
        const int f = idx / N1, j = idx % N1;
        const int sd = a.esd[(size_t)f * Kp + ec[e]];
        const bool right = sd & 1;
        foff[p][e] = (sd >> 1) * (N1 * N) + (right ? (N1 - 1 - j) : j) * N;
        fsg[p][e] = right ? 0ll : (long long)0x8000000000000000ull;
      } else {
        foff[p][e] = 0;
        fsg[p][e] = 0ll;
      }
    }
#pragma unroll
  for (int p = 0; p < PF; p++)
#pragma unroll
    for (int e = 0; e < 2; e++)
      if (kPrefetch && p * 4 + t < NF) prefetch_l1(a.Fh + foff[p][e]);  // read in the projection

  // ---- fluxes folded with the metric -> gh ----
  const double *geo = a.geo;
  double sc[2];
  {
    const double dt = *a.dtp;
#pragma unroll
    for (int e = 0; e < 2; e++) sc[e] = a.cc * dt * geo[4 * (size_t)Kp + ec[e]];
  }
#pragma unroll
  for (int e = 0; e < 2; e++) {
    const double xr = geo[ec[e]], yr = geo[(size_t)Kp + ec[e]];
    const double xs = geo[2 * (size_t)Kp + ec[e]], ys = geo[3 * (size_t)Kp + ec[e]];
#pragma unroll
    for (int p = 0; p < PQ; p++) {
      double u[N], gr[N], gs[N];
#pragma unroll
      for (int n = 0; n < N; n++) u[n] = gh[gh_slot<N>(n, p, e, 0) + lane];
      folded_flux<Eq>(q, u, xr, yr, xs, ys, gr, gs);
      const bool real = p * 4 + t < NQ;
#pragma unroll
      for (int n = 0; n < N; n++) {
        gh[gh_slot<N>(n, p, e, 0) + lane] = real ? gr[n] : 0.0;
        gh[gh_slot<N>(n, p, e, 1) + lane] = real ? gs[n] : 0.0;
      }
    }
  }

  // ---- per variable: projection, surface, RK combination, traces -> ub ----
#pragma unroll 1
  for (int n = 0; n < N; n++) {
    // this variable's stage input and u^n for the RK combination
#pragma unroll
    for (int e = 0; e < 2; e++)
#pragma unroll
      for (int p = 0; p < PM; p++)
        if (kPrefetch && p * 4 + t < NP) {
          const size_t o = (size_t)(n * NP + p * 4 + t) * Kp + ec[e];
          prefetch_l1(us + o);
          if (a.ca != 0.0) prefetch_l1(a.un + o);
        }
    double R[PM][2];
    {  // volume (K blocks GR, GS over the area points) and surface (K block E
       // over the edge points) into one accumulator when the exactness
       // bound allows it (7 * 36 * 2^14 < 2^22), else two
      // p = 3: one copy of the slicing and MMAs for the
      // three K blocks, rolled; elsewhere three unrolled copies measure faster
      if constexpr (P == 3) {
        // K block kb's input at position p of row e: g, h (kb = 0, 1) from the
        // staging slots, the side fluxes (kb = 2: -F on a left face, +F on a
        // right face) from L1
        auto xin = [&](int kb, int e, int p) -> double {
          if (kb < 2) return p < PQ ? gh[gh_slot<N>(n, p < PQ ? p : 0, e, kb) + lane] : 0.0;
          return (p < PF && p * 4 + t < NF)
                     ? __longlong_as_double(fsg[p < PF ? p : 0][e] ^
                                            __double_as_longlong(a.Fh[foff[p < PF ? p : 0][e] + n]))
                     : 0.0;
        };
        constexpr bool kMerge = 2 * NQ + NF <= 36;
        int m[2], mf[2];
  #pragma unroll
        for (int e = 0; e < 2; e++) {
          int mv = 0, ms = 0;
  #pragma unroll
          for (int p = 0; p < 4; p++) {
            mv = max(mv, max(bexp(xin(0, e, p)), bexp(xin(1, e, p))));
            ms = max(ms, bexp(xin(2, e, p)));
          }
          if (kMerge) mv = max(mv, ms);
          m[e] = quad_max(mv);
          mf[e] = kMerge ? m[e] : quad_max(ms);
        }
        long long Y[2][4];
        acc.reset();
        // one copy of the slicing and the MMAs for the three K blocks where
        // they share the MMA shape (keeps the loop body in the instruction
        // cache)
        constexpr bool kSameShape = (PQ <= 2) == (PF <= 2);
  #pragma unroll 1
        for (int kb = 0; kb < 3; kb++) {
          if (kb == 2 && !kMerge) {
  #pragma unroll
            for (int p = 0; p < PM; p++)
  #pragma unroll
              for (int e = 0; e < 2; e++)
                R[p][e] = recombine(acc, p >> 1, 2 * e + (p & 1), m[e], ozt->colexp[kProj][slot_of(p, t)]);
            acc.reset();
          }
  #pragma unroll
          for (int e = 0; e < 2; e++)
  #pragma unroll
            for (int p = 0; p < 4; p++) Y[e][p] = to_fixed(xin(kb, e, p), max(kb == 2 ? mf[e] : m[e], 1));
          if (kSameShape || kb < 2)
            contract<3, (PM + 1) / 2, (PQ <= 2)>(acc, Y, W + word_off(kProj), kb, lane);
          else
            contract<3, (PM + 1) / 2, (PF <= 2)>(acc, Y, W + word_off(kProj), kb, lane);
        }
  #pragma unroll
        for (int p = 0; p < PM; p++)
  #pragma unroll
          for (int e = 0; e < 2; e++) {
            const double v = recombine(acc, p >> 1, 2 * e + (p & 1), mf[e], ozt->colexp[kProj][slot_of(p, t)]);
            R[p][e] = kMerge ? v : R[p][e] + v;
          }
      } else {
        double xg[2][4], xh[2][4], xf[2][4];
  #pragma unroll
        for (int e = 0; e < 2; e++)
  #pragma unroll
          for (int p = 0; p < 4; p++) {
            xg[e][p] = p < PQ ? gh[gh_slot<N>(n, p < PQ ? p : 0, e, 0) + lane] : 0.0;
            xh[e][p] = p < PQ ? gh[gh_slot<N>(n, p < PQ ? p : 0, e, 1) + lane] : 0.0;
            xf[e][p] = (p < PF && p * 4 + t < NF)
                           ? __longlong_as_double(fsg[p < PF ? p : 0][e] ^
                                                  __double_as_longlong(a.Fh[foff[p < PF ? p : 0][e] + n]))
                           : 0.0;
          }
        constexpr bool kMerge = 2 * NQ + NF <= 36;
        int m[2], mf[2];
  #pragma unroll
        for (int e = 0; e < 2; e++) {
          int mv = 0, ms = 0;
  #pragma unroll
          for (int p = 0; p < 4; p++) {
            mv = max(mv, max(bexp(xg[e][p]), bexp(xh[e][p])));
            ms = max(ms, bexp(xf[e][p]));
          }
          if (kMerge) mv = max(mv, ms);
          m[e] = quad_max(mv);
          mf[e] = kMerge ? m[e] : quad_max(ms);
        }
        long long Y[2][4];
        acc.reset();
  #pragma unroll
        for (int e = 0; e < 2; e++)
  #pragma unroll
          for (int p = 0; p < 4; p++) Y[e][p] = to_fixed(xg[e][p], max(m[e], 1));
        contract<3, (PM + 1) / 2, (PQ <= 2)>(acc, Y, W + word_off(kProj), 0, lane);
  #pragma unroll
        for (int e = 0; e < 2; e++)
  #pragma unroll
          for (int p = 0; p < 4; p++) Y[e][p] = to_fixed(xh[e][p], max(m[e], 1));
        contract<3, (PM + 1) / 2, (PQ <= 2)>(acc, Y, W + word_off(kProj), 1, lane);
        if (!kMerge) {
  #pragma unroll
          for (int p = 0; p < PM; p++)
  #pragma unroll
            for (int e = 0; e < 2; e++)
              R[p][e] = recombine(acc, p >> 1, 2 * e + (p & 1), m[e], ozt->colexp[kProj][slot_of(p, t)]);
          acc.reset();
        }
  #pragma unroll
        for (int e = 0; e < 2; e++)
  #pragma unroll
          for (int p = 0; p < 4; p++) Y[e][p] = to_fixed(xf[e][p], max(mf[e], 1));
        contract<3, (PM + 1) / 2, (PF <= 2)>(acc, Y, W + word_off(kProj), 2, lane);
  #pragma unroll
        for (int p = 0; p < PM; p++)
  #pragma unroll
          for (int e = 0; e < 2; e++) {
            const double v = recombine(acc, p >> 1, 2 * e + (p & 1), mf[e], ozt->colexp[kProj][slot_of(p, t)]);
            R[p][e] = kMerge ? v : R[p][e] + v;
          }
      }
    }
    // RK combination (element_body's epilogue)
    double cnew[2][4];
#pragma unroll
    for (int e = 0; e < 2; e++)
#pragma unroll
      for (int p = 0; p < 4; p++) {
        const int idx = p * 4 + t;
        cnew[e][p] = 0.0;
        if (p < PM && idx < NP) {
          const size_t o = (size_t)(n * NP + idx) * Kp + ec[e];
          const double cin = (badv[e] && idx > 0) ? 0.0 : us[o];
          double v = fma(sc[e], R[p < PM ? p : 0][e], a.cb * cin);
          if (a.ca != 0.0) v = fma(a.ca, a.un[o], v);
          // LIM: mode 0 is the mean k_means stored, which the neighbours'
          // limiters read (the same value up to the rounding of its sum)
          if (LIM && idx == 0) v = a.M[(size_t)n * Kp + ec[e]];
          if (live[e]) {
            a.out[o] = v;
            if (badv[e] && idx > 0 && a.us != a.out) a.us[o] = 0.0;
          }
          cnew[e][p] = v;
        }
      }
    // LIM: modes 1 and 2 (position 0 of lanes t = 1, 2) for the limiter,
    // in a g/h slot of this variable that its traces leave free
    if constexpr (LIM && S::kStash) {
#pragma unroll
      for (int e = 0; e < 2; e++)
        gh[gh_slot<N>(n, PF >> 1, e, PF & 1) + lane] = cnew[e][0];
    }
    // next-stage edge traces
    int m[2];
    long long Y[2][4];
    split_rows(cnew, m, Y);
    acc.reset();
    contract<1, (PF + 1) / 2, (PM <= 2)>(acc, Y, W + word_off(kTrace), 0, lane);
#pragma unroll
    for (int p = 0; p < PF; p++)
#pragma unroll
      for (int e = 0; e < 2; e++)
        gh[gh_slot<N>(n, p >> 1, e, p & 1) + lane] =
            recombine(acc, p >> 1, 2 * e + (p & 1), m[e], ozt->colexp[kTrace][slot_of(p, t)]);
  }

  // the limiter, one variable per lane of each quad, after the loop above
  // (its inputs were staged by the other lanes of the quad)
  if constexpr (LIM) {
    __syncwarp();
    limit_epilogue<Eq, P>(tab, a, gh, lane, ec, el, live);
  }

  // lane t = 0 wrote each element's mode 0 to out; the flatten below reads it
  __syncwarp();
  // ---- positivity of the new traces; write them ----
  bool badt[2] = {false, false};
#pragma unroll
  for (int p = 0; p < PF; p++)
#pragma unroll
    for (int e = 0; e < 2; e++) {
      if (p * 4 + t >= NF) continue;
      double u[N];
#pragma unroll
      for (int n = 0; n < N; n++) u[n] = gh[gh_slot<N>(n, p >> 1, e, p & 1) + lane];
      badt[e] |= !Eq::physical(q, u);
    }
#pragma unroll
  for (int e = 0; e < 2; e++) {
    int b = badt[e] && (LIM || a.check);
    b |= __shfl_xor_sync(0xffffffffu, b, 1);
    b |= __shfl_xor_sync(0xffffffffu, b, 2);
    badt[e] = b != 0;
  }
#pragma unroll
  for (int e = 0; e < 2; e++) {
    if (!live[e]) continue;
    double *Te = a.T + (size_t)el[e] * (NF * N);
    double c0[N];
    if (badt[e]) {  // the element mean, as written to out above
#pragma unroll
      for (int n = 0; n < N; n++) c0[n] = a.out[(size_t)(n * NP) * Kp + el[e]];
    }
#pragma unroll
    for (int p = 0; p < PF; p++) {
      const int idx = p * 4 + t;
      if (idx >= NF) continue;
      const int f = idx / N1, j = idx % N1;
      double v[N];
#pragma unroll
      for (int n = 0; n < N; n++)
        v[n] = badt[e] ? c0[n] * tab.E[f][j][0] : gh[gh_slot<N>(n, p >> 1, e, p & 1) + lane];
      store_vars<N>(Te + idx * N, v);  // 128-bit stores
    }
  }
  if (badt[0] || badt[1]) {
#pragma unroll
    for (int e = 0; e < 2; e++) {
      if (!live[e] || !badt[e]) continue;
#pragma unroll
      for (int n = 0; n < N; n++)
#pragma unroll
        for (int p = 0; p < PM; p++) {
          const int idx = p * 4 + t;
          if (idx >= 1 && idx < NP) a.out[(size_t)(n * NP + idx) * Kp + el[e]] = 0.0;
        }
    }
  }
}

// Edge traces of a state with the tensor-core trace contraction (trace_body's
// rules: a non-physical trace flattens the element -- higher modes to zero,
// traces to the mean).  Bit for bit the traces k_element_oz writes for the
// same coefficients, so a run that starts from a stored state continues
// exactly as an uninterrupted one.
template <class Eq, int P>
__global__ void __launch_bounds__(kOzThreads) k_trace_oz(const __grid_constant__ Tab<P> tab,
                                                         const __grid_constant__ EqP q,
                                                         double *u, double *__restrict__ T, int K,
                                                         int Kp, const Tabs *__restrict__ ozt) {
  using S = OzShape<Eq, P>;
  constexpr int N = S::N, NP = S::NP, N1 = S::N1, NF = S::NF, PM = S::PM, PF = S::PF;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, t = lane & 3;
  const int e0 = (blockIdx.x * 4 + warp) * 16 + (lane >> 2);
  const int el[2] = {e0, e0 + 8};
  const bool live[2] = {el[0] < K, el[1] < K};
  const int ec[2] = {live[0] ? el[0] : K - 1, live[1] ? el[1] : K - 1};
  Acc acc;
  double Tv[N][PF][2];
#pragma unroll
  for (int n = 0; n < N; n++) {
    double x[2][4];
#pragma unroll
    for (int e = 0; e < 2; e++)
#pragma unroll
      for (int p = 0; p < 4; p++) {
        const int idx = p * 4 + t;
        x[e][p] = (p < PM && idx < NP) ? u[(size_t)(n * NP + idx) * Kp + ec[e]] : 0.0;
      }
    int m[2];
    long long Y[2][4];
    split_rows(x, m, Y);
    acc.reset();
    contract<1, (PF + 1) / 2, (PM <= 2)>(acc, Y, ozt->w + word_off(kTrace), 0, lane);
#pragma unroll
    for (int p = 0; p < PF; p++)
#pragma unroll
      for (int e = 0; e < 2; e++)
        Tv[n][p][e] = recombine(acc, p >> 1, 2 * e + (p & 1), m[e], ozt->colexp[kTrace][slot_of(p, t)]);
  }
  bool bad[2] = {false, false};
#pragma unroll
  for (int p = 0; p < PF; p++)
#pragma unroll
    for (int e = 0; e < 2; e++) {
      if (p * 4 + t >= NF) continue;
      double v[N];
#pragma unroll
      for (int n = 0; n < N; n++) v[n] = Tv[n][p][e];
      bad[e] |= !Eq::physical(q, v);
    }
#pragma unroll
  for (int e = 0; e < 2; e++) {
    int b = bad[e];
    b |= __shfl_xor_sync(0xffffffffu, b, 1);
    b |= __shfl_xor_sync(0xffffffffu, b, 2);
    bad[e] = b != 0;
  }
#pragma unroll
  for (int e = 0; e < 2; e++) {
    if (!live[e]) continue;
    double *Te = T + (size_t)el[e] * (NF * N);
    double c0[N];
    if (bad[e]) {
#pragma unroll
      for (int n = 0; n < N; n++) c0[n] = u[(size_t)(n * NP) * Kp + el[e]];
    }
#pragma unroll
    for (int p = 0; p < PF; p++) {
      const int idx = p * 4 + t;
      if (idx >= NF) continue;
      const int f = idx / N1, j = idx % N1;
      double v[N];
#pragma unroll
      for (int n = 0; n < N; n++) v[n] = bad[e] ? c0[n] * tab.E[f][j][0] : Tv[n][p][e];
      store_vars<N>(Te + idx * N, v);
    }
  }
  if (bad[0] || bad[1]) {
#pragma unroll
    for (int e = 0; e < 2; e++) {
      if (!live[e] || !bad[e]) continue;
#pragma unroll
      for (int n = 0; n < N; n++)
#pragma unroll
        for (int p = 0; p < PM; p++) {
          const int idx = p * 4 + t;
          if (idx >= 1 && idx < NP) u[(size_t)(n * NP + idx) * Kp + el[e]] = 0.0;
        }
    }
  }
}

// host: the f16 digit words and column exponents of the four tables
template <int P>
void build_tabs(const Tab<P> &tb, Tabs *out, double *dense);

}  // namespace oz
}  // namespace dg
