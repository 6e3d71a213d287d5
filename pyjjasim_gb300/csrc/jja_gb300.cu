// GB300 (sm_103a) RCSJ time-stepping kernels and the C ABI of libjja_gb300.so.
//
// One time step of the reference (pyjjasim time_evolution.py:523-580), for W problems at once:
//   k_junction : x = sigma*xi - Is + Ic sin(sum_k e_k theta_k) + sum_k c_k theta_k   (:533-558)
//   k_face_rhs : b = A (x/c0 - theta_s) - 2 pi f, written in the factor's face order (:560-569)
//   k_fwd_level: forward supernodal solve, one launch per elimination-tree level
//   k_bwd_level: backward supernodal solve, one launch per level (reverse order)
//   k_update   : y = A^T J ; theta_next = (y - x)/c0 ; I = y + Is ; theta_s += Vs dt  (:570-580)
// Layout: every (N, W) array is row-major with the problem index w contiguous, so a warp
// reads 32 problems of one junction/face in one 256-byte transaction when W >= 32.
#include "../../include/jja_gb300.h"
#include "jja_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <mutex>
#include <map>
#include <vector>

namespace {

thread_local std::string g_err;
std::atomic<int64_t> g_launches{0};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define JJA_CUDA(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      throw Error(JJA_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));            \
  } while (0)

template <class F>
int guarded(F&& f) {
  try {
    f();
    return JJA_OK;
  } catch (const Error& e) {
    g_err = e.what();
    return e.code;
  } catch (const std::exception& e) {
    g_err = e.what();
    return JJA_ERR_INTERNAL;
  }
}

#ifndef JJA_WARPS_PER_BLOCK
#define JJA_WARPS_PER_BLOCK 4
#endif
// Compile-time shape of the level kernels (measured on GB300: 4 warps per block and 2 columns in
// flight are best or tied on every workload; 8 warps per block costs 4 % at W = 512, an unroll
// of 4 or 8 costs 6-15 % on the small-W and ragged paths, whose supernodes are narrow).
#ifndef JJA_UNROLL
#define JJA_UNROLL 2
#endif
constexpr int kWarpsPerBlock = JJA_WARPS_PER_BLOCK;   // level kernels: one warp per work item
// rows of a work item handled by one lane (1, 2, 4 or 8). Measured on GB300: 1 and 2 tie at
// W = 512 (1.60 ms/step), 1 is 10-12 % faster than 2 for W = 1 and ragged batches, whose
// supernodes are narrow; 4 and 8 are slower everywhere.
constexpr int kDefaultRowsPerLane = 1;
constexpr int kDefaultRowsPerLaneFwdWide = 2;   // the forward sweep's default for W >= 256
constexpr int kDefaultPackRows = 24;   // W = 1: supernodes of at most this many rows go one per lane
constexpr int kPackMaxK = 8;           // ... and at most this many columns
constexpr int kPackLanesWarps = 4096;  // ... 4 lanes each on levels with fewer one-lane pack warps
constexpr int kDefaultPackMinWarps = 152 * 32;   // ... on levels whose regular items need this many warps
constexpr int kGroupsFromW = 256;      // from this many problems the step runs as concurrent groups ...
constexpr int kGroupW = 160;           // ... of about this many problems, 2 to 4 of them
constexpr int kNumSMs = 152;                     // GB300
constexpr int kDefaultTargetWarps = 152 * 24;   // levels with fewer work items split their dot products
constexpr int kDefaultTargetWarpsSmallW = 152 * 64;   // ... for 2-16 problems
constexpr int kFwdWideFaces = 1 << 17;          // forward sweep: two rows per lane from W = 8 on this many faces
constexpr int kDefaultMinPiece = 16;     // shortest piece of a split dot product
constexpr int kDefaultSubRows = 32;     // subtree sweeps: rows per subtree (columns + the root's off-diagonal rows)
constexpr int kSubMaxRows = 64;          // ... at most this many rows (tuning bound)
constexpr int kDefaultSubRows1 = 16;     // ... at W = 1 (subtree packs of 32 subtrees)
constexpr int kSubPackMinWarps = 152 * 4;   // ... where the packs fill at least this many warps
constexpr int kSubMinWarps = 152 * 16;  // ... by default only when the launch has at least this many warps
constexpr int kSubMaxWarps = 8;         // ... warps (32-problem blocks of one subtree) per block
constexpr int kSubMaxK = 8;             // ... members of at most this many columns
constexpr int kSubMaxF = 2048;          // ... at most this many F values per subtree
constexpr int kSubMaxL = 4096;          // ... at most this many off-diagonal entries per subtree
constexpr int kUnroll = JJA_UNROLL;   // columns whose loads are issued ahead of their FMAs
constexpr double kTwoPi = 6.283185307179586;
constexpr int kEllMax = 6;          // faces with up to 6 junctions (square 4, triangular 3, honeycomb 6)

// ------------------------------------------------------------------------------------------
// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC 2011), used for on-device thermal noise.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += W0;
    k.y += W1;
  }
  return c;
}

// one standard normal per (element, step) via Box-Muller in single precision; noise values
// need no FP64 accuracy and GB300's FP32 pipe is far wider than its FP64 pipe
__device__ __forceinline__ double philox_normal(uint64_t seed, uint64_t elem, uint64_t step) {
  uint4 c = make_uint4((uint32_t)elem, (uint32_t)(elem >> 32), (uint32_t)step, (uint32_t)(step >> 32));
  uint4 r = philox4x32_10(c, make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  const float u1 = ((float)(r.x >> 8) + 1.0f) * (1.0f / 16777216.0f);  // (0, 1]
  const float u2 = (float)(r.y >> 8) * (1.0f / 16777216.0f);           // [0, 1)
  const float rad = sqrtf(-2.0f * logf(u1));
  return (double)(rad * cospif(2.0f * u2));
}

// Programmatic dependent launch: every kernel first lets the next kernel of its stream be
// scheduled (once all of its own blocks have started), then waits until the previous kernel
// has finished and its writes are visible. The dependent launch overlaps the ~us gap between
// the many short kernels of a step; both instructions are no-ops for plain launches.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
}

// value of a source at (n, w) in time slot tt = step - window start (ignored when stride_t == 0)
__device__ __forceinline__ double view_at(const jja_view& v, int64_t n, int64_t w, int64_t tt = 0) {
  return v.ptr ? __ldg(v.ptr + n * v.stride_n + w * v.stride_w + tt * v.stride_t) : 0.0;
}

struct StepArgs {
  int Nj, Nf, W, width;
  int w0, wn;          // the launch steps problems [w0, w0 + wn) of the W in the arrays (a group)
  const double* h[4];
  double* hout;
  double* theta_s;
  jja_view Is, f, Vs, T;
  int noise_mode;
  const double* noise;
  uint64_t seed;
  // device counters: [0] step whose face RHS comes next (written by k_update), [1] that step + 1
  // (written by k_face_rhs), [2] first step of the time-dependent source window, [3] first step
  // of the call. Each kernel writes only a slot that no other thread of the same launch reads.
  int64_t* d_step;
  int64_t th_slot, I_slot;
  int store_all;       // every step of the call is stored, at slot (step - first step of the call)
  double* th_out;
  double* I_out;
  double e[4];
  double dt;
  jja_view Isq;        // Is / c0 for a time-independent Is (plan-owned, refreshed at the start of a run)
  int resistive;       // width 3 and no capacitance anywhere: c1 / c0 = -1, c2 = 0
};

struct Tables {
  const double* Icq;    // Ic / c0: Nj values, or Nj x W when critical currents differ per problem
  const double* Ic;     // Ic, same layout (the adjoint needs it unscaled)
  int ic_per_w;         // 1: Icq / Ic are (Nj x W)
  const double* inv_c0;
  const double* coefq;  // (width-1) x Nj: c_k / c0
  const double* coef;   // (width-1) x Nj: c_k
  const double* Rvq;    // Rv / c0^2 (noise amplitude over c0 is sqrt(2 T Rvq))
  const int64_t* fj_ptr;   // permuted face -> junction entries
  const int32_t* fj_col;
  const int32_t* face_orig;
  const int32_t* fj_ell;   // faces of <= kEllMax junctions: Nf x face_deg codes, padded with -1
  int face_deg;            // 0 when some face has more than kEllMax junctions (CSR path)
  const int32_t* jf_face;  // 2 per junction: (permuted face << 1) | (A entry is -1), or -1
  const longlong2* sincos; // per k < 65536: {S, C} = {sin, cos}(k pi/32768) in units of 2^-62
  int* nonfinite;          // set to 1 by k_update when a new phase is NaN or +-inf (read by jja_plan_check)
};

// NaN or +-inf: all exponent bits set (an integer test, no FP64 instruction)
__device__ __forceinline__ bool non_finite(double v) {
  return ((unsigned)__double2hiint(v) & 0x7ff00000u) == 0x7ff00000u;
}

// +-v by flipping the sign bit (no FP64 instruction)
__device__ __forceinline__ double signed_by(double v, int neg) {
  return __hiloint2double(__double2hiint(v) ^ (neg << 31), __double2loint(v));
}

// ------------------------------------------------------------------------------------------
// sin(x) and cos(x) to FP64 accuracy without FP64 instructions. GB300's FP64 pipe is ~60x
// narrower than its FP32 and integer pipes, and the junction kernels are bound by it; this
// evaluation runs on the integer pipe (64-bit fixed point) with an FP32 correction term.
// Table-driven method (Tang, ACM TOMS 15(2), 1989) with an exact Payne-Hanek style reduction:
// 1. |x| = M 2^(e-1075) exactly (M: the 53-bit significand). u = |x| 2^15/pi is formed as M times
//    2^15/pi held to 128 bits (kInvPiHi:kInvPiLo = floor(2^129/pi), computed to 400 bits with
//    mpmath), keeping 64 fractional bits of u and the low bits of its integer part (error
//    < |x| 2^-114 in u: below 2^-70 for the phases' range, 2^-52 at |x| = 2^62). k = nearest
//    integer to u, f = u - k in [-1/2, 1/2], t = f pi/2^15 (|t| <= 4.8e-5) as a signed 64-bit
//    number in units of 2^-76 (kPi61 = round(pi 2^61)).
// 2. With S, C = sin, cos(k pi/32768) from a 65536-entry table in units of 2^-62 (1 MB,
//    L2-resident, computed on the host in extended precision):
//      sin(|x|) = S + C t - S t^2/2 - C t^3/6,   cos(x) = C - S t - C t^2/2 + S t^3/6,
//    remainder below 3e-19. S + C t and the quadratic term are formed in fixed point (64x64-bit
//    products), the cubic term (< 1.9e-14) in FP32 (absolute error < 2e-21).
// 3. The fixed-point sum (absolute error ~1e-18) is rounded to the nearest double with integer
//    operations (count of leading zeros, shift, round half to even).
// |x| < 2^-27 gives sin = x, cos = 1 (the next terms are below half an ulp); |x| >= 2^62, inf
// and NaN give NaN. No library call: the kernels keep no stack frame for one. Host and device
// share this code, so the library can check it on the CPU (jja_sin_host).
// ------------------------------------------------------------------------------------------
constexpr int kSinTable = 65536;
constexpr uint64_t kInvPiHi = 0xa2f9836e4e441529ull;   // floor(2^15/pi 2^114) = kInvPiHi 2^64 + kInvPiLo
constexpr uint64_t kInvPiLo = 0xfc2757d1f534ddc0ull;
constexpr int64_t kPi61 = 0x6487ed5110b4611all;       // round(pi 2^61)

__host__ __device__ __forceinline__ uint64_t umulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

__host__ __device__ __forceinline__ int64_t smulhi64(int64_t a, int64_t b) {
#ifdef __CUDA_ARCH__
  return __mul64hi(a, b);
#else
  return (int64_t)(((__int128)a * b) >> 64);
#endif
}

__host__ __device__ __forceinline__ uint64_t bits_of(double v) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t b;
  memcpy(&b, &v, 8);
  return b;
#endif
}

__host__ __device__ __forceinline__ double double_of(uint64_t b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double v;
  memcpy(&v, &b, 8);
  return v;
#endif
}

__host__ __device__ __forceinline__ float float_of_int(int v) {
#ifdef __CUDA_ARCH__
  return __int2float_rn(v);
#else
  return (float)v;
#endif
}

// f 2^62 truncated to an integer, for |f| < 2^-28 (the cubic terms)
__host__ __device__ __forceinline__ int64_t fixed62_of_float(float f) {
  uint32_t b;
#ifdef __CUDA_ARCH__
  b = __float_as_uint(f);
#else
  memcpy(&b, &f, 4);
#endif
  const int E = (int)((b >> 23) & 0xffu);
  const int64_t m = (int64_t)((b & 0x7fffffu) | 0x800000u);
  const int sh = E - 88;   // f 2^62 = m 2^(E - 150 + 62)
  const int64_t v = E == 0 ? 0 : sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0);
  return (b >> 31) ? -v : v;
}

// R 2^-62 rounded to the nearest double, negated when `neg`
__host__ __device__ __forceinline__ double double_of_fixed62(int64_t R, bool neg) {
  const bool sign = (R < 0) != neg;
  const uint64_t a = R < 0 ? (uint64_t)0 - (uint64_t)R : (uint64_t)R;
  if (a == 0) return double_of((uint64_t)neg << 63);
#ifdef __CUDA_ARCH__
  const int lz = __clzll((long long)a);
#else
  const int lz = __builtin_clzll(a);
#endif
  const uint64_t n = a << lz;                     // leading one at bit 63
  uint64_t mant = n >> 11;                        // 53 bits
  const uint64_t rem = n & 0x7ffu;
  mant += (rem > 0x400u) || (rem == 0x400u && (mant & 1u));
  // value in [2^(1-lz), 2^(2-lz)): biased exponent 1024 - lz; a carry out of the rounding
  // moves into the exponent field
  return double_of((((uint64_t)(1023 - lz) << 52) + mant) | ((uint64_t)sign << 63));
}

struct SinReduced {
  unsigned idx;    // k mod 65536
  int64_t t;       // t in units of 2^-76
};

// 64 bits of the 192-bit number (P2 P1 P0) starting at bit `pos` (0 <= pos), zeros above bit 191
__host__ __device__ __forceinline__ uint64_t bits_at(uint64_t P0, uint64_t P1, uint64_t P2, int pos) {
  if (pos >= 192) return 0;
  if (pos >= 128) return P2 >> (pos - 128);
  if (pos == 64) return P1;
  if (pos > 64) return (P1 >> (pos - 64)) | (P2 << (128 - pos));
  if (pos == 0) return P0;
  return (P0 >> pos) | (P1 << (64 - pos));
}

// step 1 for 2^-27 <= |x| < 2^62 (biased exponent e in [996, 1084])
__host__ __device__ __forceinline__ SinReduced sin_reduce(uint64_t ax) {
  const int e = (int)(ax >> 52);
  const uint64_t M = (ax & 0xfffffffffffffull) | (1ull << 52);
  // P = M (kInvPiHi 2^64 + kInvPiLo), 181 bits
  const uint64_t P0 = M * kInvPiLo, a_hi = umulhi64(M, kInvPiLo);
  const uint64_t b_lo = M * kInvPiHi, b_hi = umulhi64(M, kInvPiHi);
  const uint64_t P1 = a_hi + b_lo;
  const uint64_t P2 = b_hi + (P1 < a_hi ? 1u : 0u);
  // u 2^64 = P 2^(e - 1125): fraction = bits [sh, sh + 64) of P, integer part above (only its
  // low 16 bits index the table)
  const int sh = 1125 - e;   // 41 .. 129
  const uint64_t frac = bits_at(P0, P1, P2, sh);
  const uint64_t kint = bits_at(P0, P1, P2, sh + 64);
  SinReduced r;
  r.idx = (unsigned)(kint + (frac >> 63)) & (unsigned)(kSinTable - 1);   // round to nearest
  r.t = smulhi64((int64_t)frac, kPi61);   // f 2^64 pi 2^61 2^-64 = t 2^76
  return r;
}

// steps 2 and 3: sin(|x|) and cos(x) from the reduction and the table entry {S, C} (2^-62
// units). t^2 is formed in units of 2^-88; the cubic term (< 1.9e-14) in FP32.
__host__ __device__ __forceinline__ int64_t sin_fixed(const SinReduced& r, longlong2 sc) {
  const int64_t ct = (smulhi64(sc.y, r.t) + (1 << 11)) >> 12;         // C t
  const int64_t t2 = smulhi64(r.t, r.t);                               // t^2 2^88
  const int64_t st2 = (smulhi64(sc.x, t2) + (1 << 24)) >> 25;          // S t^2 / 2
  const float tf = float_of_int((int)(r.t >> 32)) * 0x1p-44f, cf = float_of_int((int)(sc.y >> 32)) * 0x1p-30f;
  const float cubic = (-(1.0f / 6.0f) * cf) * (tf * tf * tf);          // -C t^3/6
  return sc.x + ct - st2 + fixed62_of_float(cubic);
}

__host__ __device__ __forceinline__ int64_t cos_fixed(const SinReduced& r, longlong2 sc) {
  const int64_t st = (smulhi64(sc.x, r.t) + (1 << 11)) >> 12;         // S t
  const int64_t t2 = smulhi64(r.t, r.t);
  const int64_t ct2 = (smulhi64(sc.y, t2) + (1 << 24)) >> 25;          // C t^2 / 2
  const float tf = float_of_int((int)(r.t >> 32)) * 0x1p-44f, sf = float_of_int((int)(sc.x >> 32)) * 0x1p-30f;
  const float cubic = ((1.0f / 6.0f) * sf) * (tf * tf * tf);           // S t^3/6
  return sc.y - st - ct2 + fixed62_of_float(cubic);
}

__host__ __device__ __forceinline__ longlong2 sin_table_entry(const longlong2* tab, unsigned idx) {
#ifdef __CUDA_ARCH__
  return __ldg(tab + idx);
#else
  return tab[idx];
#endif
}

// |x| >= 2^62 (where x carries no information modulo 2 pi), inf and NaN give NaN
__host__ __device__ __forceinline__ bool sin_outside_range(uint64_t ax) { return ax >= (1085ull << 52); }
__host__ __device__ __forceinline__ bool sin_tiny(uint64_t ax) { return ax < (996ull << 52); }   // |x| < 2^-27
constexpr uint64_t kNaNBits = 0x7ff8000000000000ull;

__host__ __device__ __forceinline__ double fast_sin(double x, const longlong2* __restrict__ tab) {
  const uint64_t xb = bits_of(x), ax = xb & 0x7fffffffffffffffull;
  if (sin_outside_range(ax)) return double_of(kNaNBits);
  if (sin_tiny(ax)) return x;
  const SinReduced r = sin_reduce(ax);
  return double_of_fixed62(sin_fixed(r, sin_table_entry(tab, r.idx)), (xb >> 63) != 0);
}

__host__ __device__ __forceinline__ void fast_sincos(double x, const longlong2* __restrict__ tab, double& s_out,
                                                     double& c_out) {
  const uint64_t xb = bits_of(x), ax = xb & 0x7fffffffffffffffull;
  if (sin_outside_range(ax)) {
    s_out = c_out = double_of(kNaNBits);
    return;
  }
  if (sin_tiny(ax)) {
    s_out = x;
    c_out = 1.0;
    return;
  }
  const SinReduced r = sin_reduce(ax);
  const longlong2 sc = sin_table_entry(tab, r.idx);
  s_out = double_of_fixed62(sin_fixed(r, sc), (xb >> 63) != 0);
  c_out = double_of_fixed62(cos_fixed(r, sc), false);
}

// q(j, w) = x / c0 for the step whose phase history is th[0..] (time_evolution.py:533-558):
//   x = sqrt(2 T Rv) xi - Is + Ic sin(sum_k e_k th_k) + sum_k c_k th_k
// evaluated with the coefficients already divided by c0 (Icq = Ic/c0, coefq_k = c_k/c0,
// Rvq = Rv/c0^2, Isq = Is/c0), which saves the final multiply. Without capacitance
// (stencil width 3) c1/c0 = -1 and c2 = 0 exactly, so x/c0 = Icq sin - th1 - Isq.
// `step` keys the Philox stream; tt = step - window start indexes time-dependent sources.
__device__ __forceinline__ double junction_q(const StepArgs& a, const Tables& t, int64_t e, int64_t j, int64_t w,
                                            const double* th, int64_t step, int64_t tt) {
  double arg;
  if (a.width == 3) {
    arg = fma(2.0, th[0], -th[1]);        // 2 th1 - th2 with the reference's single rounding
  } else {
    arg = a.e[0] * th[0];
#pragma unroll
    for (int k = 1; k < 4; ++k)
      if (k < a.width - 1) arg = fma(a.e[k], th[k], arg);
  }
  const double s = fast_sin(arg, t.sincos);
  const double icq = __ldg(t.Icq + (t.ic_per_w ? e : j));
  double X;
  if (a.resistive) {
    X = fma(icq, s, -th[0]);
  } else {
    X = icq * s;
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (k < a.width - 1) X = fma(__ldg(t.coefq + (int64_t)k * a.Nj + j), th[k], X);
  }
  // Is / c0: precomputed when Is does not change with time, else scaled here
  const double isq = a.Isq.ptr ? view_at(a.Isq, j, w) : view_at(a.Is, j, w, tt) * __ldg(t.inv_c0 + j);
  if (a.noise_mode == JJA_NOISE_NONE)
    return a.Is.ptr ? X - isq : X;   // (0 - Is) + X in the reference
  const double T = view_at(a.T, j, w, tt);
  const double xi = a.noise_mode == JJA_NOISE_BUFFER ? a.noise[e] : philox_normal(a.seed, (uint64_t)e, (uint64_t)step);
  const double fl = sqrt(2.0 * T * __ldg(t.Rvq + j)) * xi;
  return (fl - isq) + X;
}

// Isq = Is / c0 per junction, refreshed at the start of every run (and every host-driven step)
__global__ void __launch_bounds__(256) k_scale_sources(jja_view Is, const double* __restrict__ inv_c0,
                                                       double* __restrict__ Isq, int Nj, int W) {
  pdl_begin();
  const int64_t NjW = (int64_t)Nj * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < NjW; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / W, w = e - j * W;
    Isq[e] = view_at(Is, j, w) * __ldg(inv_c0 + j);
  }
}

// q for the first step of a run, from the stored phase history
__global__ void __launch_bounds__(256) k_junction(StepArgs a, Tables t, double* __restrict__ q) {
  pdl_begin();
  const int64_t n = (int64_t)a.Nj * a.wn;
  const int64_t step = a.d_step[0], tt = step - a.d_step[2];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i / a.wn, w = a.w0 + (i - j * a.wn), e = j * a.W + w;
    double th[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) th[k] = (k < a.width - 1) ? a.h[k][e] : 0.0;
    q[e] = junction_q(a, t, e, j, w, th, step, tt);
  }
}

// the step counters at the start of a call (kernel arguments are fixed at launch, so the
// host's values need no pinned staging)
__global__ void k_set_counters(int64_t* __restrict__ d_step, int64_t step, int64_t t0) {
  pdl_begin();
  d_step[0] = step;
  d_step[1] = step;
  d_step[2] = t0;
  d_step[3] = step;   // first step of the call: output slot 0 when every step is stored
}

// b(p, w) = sum_j A_pj (q_j - theta_s_j) - 2 pi f_p, p in the factor's face order. Also
// publishes step + 1 in d_step[1] (read by k_update, which evaluates the next step's q).
__global__ void __launch_bounds__(256) k_face_rhs(StepArgs a, Tables t, const double* __restrict__ q,
                                                  double* __restrict__ b) {
  pdl_begin();
  const int64_t n = (int64_t)a.Nf * a.wn;
  const int64_t step = a.d_step[0], tt = step - a.d_step[2];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = i / a.wn, w = a.w0 + (i - p * a.wn), e = p * a.W + w;
    double acc = 0.0;
    if (t.face_deg) {
      // fixed-degree layout: all index loads, then all value loads, then the sum
      int code[kEllMax];
      double v[kEllMax];
#pragma unroll
      for (int d = 0; d < kEllMax; ++d) code[d] = d < t.face_deg ? __ldg(t.fj_ell + p * t.face_deg + d) : -1;
#pragma unroll
      for (int d = 0; d < kEllMax; ++d) {
        const int64_t j = code[d] >> 1;
        v[d] = code[d] >= 0 ? q[j * a.W + w] : 0.0;
        if (a.theta_s && code[d] >= 0) v[d] -= a.theta_s[j * a.W + w];
      }
      acc = signed_by(v[0], code[0] & 1);
#pragma unroll
      for (int d = 1; d < kEllMax; ++d)
        if (code[d] >= 0) acc += signed_by(v[d], code[d] & 1);
    } else {
      const int64_t i0 = __ldg(t.fj_ptr + p), i1 = __ldg(t.fj_ptr + p + 1);
      for (int64_t k = i0; k < i1; ++k) {
        const int code = __ldg(t.fj_col + k);          // (junction << 1) | (A entry is -1)
        const int64_t j = code >> 1;
        double v = q[j * a.W + w];
        if (a.theta_s) v -= a.theta_s[j * a.W + w];
        v = signed_by(v, code & 1);
        acc = (k == i0) ? v : acc + v;
      }
    }
    if (a.f.ptr) acc = fma(-kTwoPi, view_at(a.f, __ldg(t.face_orig + p), w, tt), acc);
    b[e] = acc;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.d_step[1] = step + 1;
}

// theta_next = (A^T J)/c0 - q, outputs, theta_s update (time_evolution.py:562-580); with
// `fuse_next` the same thread then evaluates q of the next step from the new history
// (theta_next, h[0], ...), saving a pass over the phase arrays.
#ifndef JJA_UPDATE_MIN_BLOCKS
#define JJA_UPDATE_MIN_BLOCKS 6   // resident blocks per SM the register allocation must allow (measured: 4 -> 6 is 16 % faster)
#endif
template <bool kFuseNext>
__global__ void __launch_bounds__(256, JJA_UPDATE_MIN_BLOCKS) k_update(StepArgs a, Tables t, double* __restrict__ q,
                                                const double* __restrict__ J) {
  pdl_begin();
  const int64_t NjW = (int64_t)a.Nj * a.W, n = (int64_t)a.Nj * a.wn;
  const int64_t next_step = a.d_step[1];            // published by this step's k_face_rhs
  const int64_t tt = next_step - 1 - a.d_step[2];   // source slot of the step being finished
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i / a.wn, w = a.w0 + (i - j * a.wn), e = j * a.W + w;
    // y = A^T J: a junction lies on one or two faces; the +-1 entries are sign flips
    const int p0 = __ldg(t.jf_face + 2 * j), p1 = __ldg(t.jf_face + 2 * j + 1);
    double y = p0 >= 0 ? signed_by(J[(int64_t)(p0 >> 1) * a.W + w], p0 & 1) : 0.0;
    if (p1 >= 0) y += signed_by(J[(int64_t)(p1 >> 1) * a.W + w], p1 & 1);
    const double th = fma(y, __ldg(t.inv_c0 + j), -q[e]);
    if (non_finite(th)) *t.nonfinite = 1;   // a diverging run is reported, not silently continued
    double hist[4];
    if (kFuseNext) {
      hist[0] = th;
#pragma unroll
      for (int k = 1; k < 4; ++k) hist[k] = (k < a.width - 1) ? a.h[k - 1][e] : 0.0;
    }
    a.hout[e] = th;
    // output slot: per step from the host, or (store_all) the step's offset in the call
    const int64_t th_slot = a.store_all ? next_step - 1 - a.d_step[3] : a.th_slot;
    const int64_t I_slot = a.store_all ? next_step - 1 - a.d_step[3] : a.I_slot;
    if (a.th_out && th_slot >= 0) a.th_out[th_slot * NjW + e] = th;
    if (a.I_out && I_slot >= 0) a.I_out[I_slot * NjW + e] = y + view_at(a.Is, j, w, tt);
    if (a.theta_s && a.Vs.ptr) a.theta_s[e] += view_at(a.Vs, j, w, tt) * a.dt;
    if (kFuseNext) q[e] = junction_q(a, t, e, j, w, hist, next_step, tt + 1);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.d_step[0] = next_step;
}

// ------------------------------------------------------------------------------------------
// supernodal triangular solves. Work item = (supernode s, output rows [r0, r1), problems
// [w0, w0+WB), contraction range [c_lo, c_hi)), packed in an int4:
//   x = s, y = r0 | r1 << 16, z = w0 | partial << 30, w = c_lo | c_hi << 16.
// Lane l handles problem w0 + l % WB and rows r0 + l / WB + t * (32 / WB), t < kRowsPerLane.
// Levels with few items split long dot products over several items ("partial" items add
// their share atomically into outputs that were zeroed at the start of the solve), so the
// top of the elimination tree has enough warps in flight to hide L2 latency.
// ------------------------------------------------------------------------------------------
struct Item {
  int s, r0, r1, w0, c_lo, c_hi;
  bool partial;
};

__device__ __forceinline__ Item unpack_item(int4 v) {
  Item it;
  it.s = v.x;
  it.r0 = v.y & 0xffff;
  it.r1 = (int)((unsigned)v.y >> 16);
  it.w0 = v.z & 0x3fffffff;
  it.partial = (v.z >> 30) & 1;
  it.c_lo = v.w & 0xffff;
  it.c_hi = (int)((unsigned)v.w >> 16);
  return it;
}

// zero the listed rows (columns [w0, w0 + wn)) of an (Nf x W) vector before a sweep whose partial items accumulate
// there, and the sweep's dataflow counters (n_ctr of them, none for level-synchronous sweeps)
__global__ void k_zero_rows(double* __restrict__ v, const int32_t* __restrict__ rows, int n_rows, int W, int w0,
                            int wn, unsigned* __restrict__ ctr, int n_ctr) {
  pdl_begin();
  const int64_t n = (int64_t)n_rows * wn;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = tid; e < n; e += nth) {
    const int64_t i = e / wn, w = w0 + (e - i * wn);
    v[(int64_t)__ldg(rows + i) * W + w] = 0.0;
  }
  for (int64_t e = tid; e < n_ctr; e += nth) ctr[e] = 0u;
}

// Load of a face-vector element that the item reads. In a level launch the rows an item reads
// are final for the whole launch (this level only writes other rows: its own outputs and, by
// atomics, its ancestors' rows), so they go through the read-only cache; in a dataflow sweep
// other warps of the same launch may just have written them, so they are read through L2.
template <bool kSharedLaunch>
__device__ __forceinline__ double load_vec(const double* p) {
  return kSharedLaunch ? __ldcg(p) : __ldg(p);
}

struct FactorDev {
  const int32_t* col0;
  const int32_t* k;
  const int32_t* m;
  const int64_t* rowptr;
  const int32_t* rows;
  const int64_t* valptr;
  const double* fcol;   // F_s column-major ((k+m) x k)
  const double* frow;   // F_s row-major
  const int4* pack_meta;     // W = 1 packs: per lane (col0, k, k + m, rowptr) of its supernode
  const double* pack_vals;   // W = 1 packs: the F_s of a pack's supernodes interleaved by lane
};

// W = 1 packs. A work item whose x field is negative covers up to 32 / LPS small supernodes of
// one level, LPS (1, 2 or 4) lanes each: pack p = -1 - x, y supernodes, z = NP | KP << 16 |
// LPS << 24 (the largest row and column count among them), w = offset of its values in units
// of 32 doubles. Lane l serves slot l / LPS (its supernode) and that supernode's rows
// r = g + LPS rr, g = l % LPS; F_s(r, j) sits at pack_vals[32 (w + j NPq + rr) + l] with
// NPq = ceil(NP / LPS), zero padded, so every load instruction of the warp reads 256
// contiguous bytes while each lane walks its rows. Levels with many more small supernodes than
// a wave of warps use them: a regular item there leaves most lanes idle and pays a chain of
// dependent loads for a handful of FMAs; more lanes per supernode give more warps and shorter
// chains per lane. KM (>= KP) sizes the register arrays.
struct PackShape {
  int count, NP, KP, LPS, NPq;
};

__device__ __forceinline__ PackShape pack_shape(const int4 raw) {
  PackShape ps;
  ps.count = raw.y;
  ps.NP = raw.z & 0xffff;
  ps.KP = (raw.z >> 16) & 0xff;
  ps.LPS = (raw.z >> 24) & 0x7;
  ps.NPq = (ps.NP + ps.LPS - 1) / ps.LPS;
  return ps;
}

template <int KM, bool kSharedLaunch>
__device__ __forceinline__ void fwd_pack(const FactorDev& F, const int4 raw, int lane, double* __restrict__ b,
                                         double* __restrict__ z) {
  const PackShape ps = pack_shape(raw);
  const int slot = lane / ps.LPS, g = lane - slot * ps.LPS;
  if (slot >= ps.count) return;
  const int4 meta = __ldg(F.pack_meta + (int64_t)(-1 - raw.x) * 32 + slot);
  const int c0 = meta.x, k = meta.y, nf = meta.z;
  const int32_t* R = F.rows + meta.w;
  // the supernode's own rows of b are final (its descendants sit on earlier levels) and no item
  // of this level writes them
  double bv[KM];
#pragma unroll
  for (int j = 0; j < KM; ++j) bv[j] = j < k ? load_vec<kSharedLaunch>(b + c0 + j) : 0.0;
  const double* V = F.pack_vals + (int64_t)raw.w * 32 + lane;
  // rows unrolled so that about 16 loads of each lane are in flight
#pragma unroll(16 / KM)
  for (int rr = 0; rr < ps.NPq; ++rr) {
    const int r = g + rr * ps.LPS;
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j < KM; ++j)
      if (j < ps.KP) acc = fma(__ldg(V + ((int64_t)j * ps.NPq + rr) * 32), bv[j], acc);
    if (r < k) z[c0 + r] = acc;
    else if (r < nf) atomicAdd(b + __ldg(R + (r - k)), -acc);
  }
}

// every lane of the warp runs this to the end (the partial sums of a supernode's lanes are
// combined with warp shuffles)
template <int KM, bool kSharedLaunch>
__device__ __forceinline__ void bwd_pack(const FactorDev& F, const int4 raw, int lane, const double* __restrict__ z,
                                         double* __restrict__ x) {
  const PackShape ps = pack_shape(raw);
  const int slot = lane / ps.LPS, g = lane - slot * ps.LPS;
  const bool active = slot < ps.count;
  int c0 = 0, k = 0, nf = 0;
  const int32_t* R = F.rows;
  if (active) {
    const int4 meta = __ldg(F.pack_meta + (int64_t)(-1 - raw.x) * 32 + slot);
    c0 = meta.x;
    k = meta.y;
    nf = meta.z;
    R = F.rows + meta.w;
  }
  const double* V = F.pack_vals + (int64_t)raw.w * 32 + lane;
  double acc[KM];
#pragma unroll
  for (int i = 0; i < KM; ++i) acc[i] = 0.0;
  // x_s = F11^T z_s - F21^T x_R: the ancestors' rows of x were written by earlier launches
#pragma unroll(16 / KM)
  for (int rr = 0; rr < ps.NPq; ++rr) {
    const int r = g + rr * ps.LPS;
    double v = 0.0;
    if (r < k) v = __ldg(z + c0 + r);
    else if (r < nf) v = -load_vec<kSharedLaunch>(x + __ldg(R + (r - k)));
#pragma unroll
    for (int i = 0; i < KM; ++i)
      if (i < ps.KP) acc[i] = fma(__ldg(V + ((int64_t)i * ps.NPq + rr) * 32), v, acc[i]);
  }
  // the LPS lanes of a slot are adjacent and aligned: butterfly sums within them
  for (int off = 1; off < ps.LPS; off <<= 1)
#pragma unroll
    for (int i = 0; i < KM; ++i) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], off);
  if (active && g == 0) {
#pragma unroll
    for (int i = 0; i < KM; ++i)
      if (i < k) x[c0 + i] = acc[i];
  }
}

template <bool kSharedLaunch>
__device__ __forceinline__ void fwd_pack_any(const FactorDev& F, const int4 raw, int lane, double* __restrict__ b,
                                             double* __restrict__ z) {
  const int KP = (raw.z >> 16) & 0xff;
  if (KP <= 2) fwd_pack<2, kSharedLaunch>(F, raw, lane, b, z);
  else if (KP <= 4) fwd_pack<4, kSharedLaunch>(F, raw, lane, b, z);
  else fwd_pack<kPackMaxK, kSharedLaunch>(F, raw, lane, b, z);
}

template <bool kSharedLaunch>
__device__ __forceinline__ void bwd_pack_any(const FactorDev& F, const int4 raw, int lane,
                                             const double* __restrict__ z, double* __restrict__ x) {
  const int KP = (raw.z >> 16) & 0xff;
  if (KP <= 2) bwd_pack<2, kSharedLaunch>(F, raw, lane, z, x);
  else if (KP <= 4) bwd_pack<4, kSharedLaunch>(F, raw, lane, z, x);
  else bwd_pack<kPackMaxK, kSharedLaunch>(F, raw, lane, z, x);
}

// One forward work item (one warp): rows [r0, r1) of F_s b_s; diagonal rows go to z, the
// off-diagonal rows are scattered (subtracted) into the ancestors' rows of b.
template <int kRowsPerLane, bool kSharedLaunch>
__device__ __forceinline__ void fwd_item(const FactorDev& F, const Item& item, int lane, int W, int WB,
                                         double* __restrict__ b, double* __restrict__ z) {
  const int s = item.s, r0 = item.r0, r1 = item.r1, w0 = item.w0;
  const int LG = 32 / WB;
  const int w = w0 + lane % WB;
  if (w >= W) return;
  const int rl = lane / WB;
  const int c0 = __ldg(F.col0 + s), k = __ldg(F.k + s), m = __ldg(F.m + s), nf = k + m;
  const double* Fs = F.fcol + __ldg(F.valptr + s);
  double acc[kRowsPerLane];
  int rr[kRowsPerLane];
#pragma unroll
  for (int t = 0; t < kRowsPerLane; ++t) {
    acc[t] = 0.0;
    const int r = r0 + rl + t * LG;
    rr[t] = r < r1 ? r : r0;
  }
  // dot products over the supernode's columns; loads of kUnroll columns are issued before
  // their FMAs so a warp keeps several L2 requests in flight (top levels have few warps)
  const int jend = min(min(k, r1), item.c_hi);
  int j = item.c_lo;
  for (; j + kUnroll <= jend; j += kUnroll) {
    double bj[kUnroll], fv[kUnroll][kRowsPerLane];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) bj[u] = load_vec<kSharedLaunch>(b + (int64_t)(c0 + j + u) * W + w);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int t = 0; t < kRowsPerLane; ++t) fv[u][t] = __ldg(Fs + (int64_t)(j + u) * nf + rr[t]);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int t = 0; t < kRowsPerLane; ++t) acc[t] = fma(fv[u][t], bj[u], acc[t]);
  }
  for (; j < jend; ++j) {
    const double bj = load_vec<kSharedLaunch>(b + (int64_t)(c0 + j) * W + w);
    const double* col = Fs + (int64_t)j * nf;
#pragma unroll
    for (int t = 0; t < kRowsPerLane; ++t) acc[t] = fma(__ldg(col + rr[t]), bj, acc[t]);
  }
  const int32_t* R = F.rows + __ldg(F.rowptr + s);
#pragma unroll
  for (int t = 0; t < kRowsPerLane; ++t) {
    const int r = r0 + rl + t * LG;
    if (r >= r1) break;
    if (r >= k) atomicAdd(b + (int64_t)__ldg(R + (r - k)) * W + w, -acc[t]);
    else if (item.partial) atomicAdd(z + (int64_t)(c0 + r) * W + w, acc[t]);
    else z[(int64_t)(c0 + r) * W + w] = acc[t];
  }
  (void)m;
}

// One backward work item: rows [i0, i1) of x_s = inv(L11)^T z_s - (L21 inv(L11))^T x[R_s].
template <int kRowsPerLane, bool kSharedLaunch>
__device__ __forceinline__ void bwd_item(const FactorDev& F, const Item& item, int lane, int W, int WB,
                                         const double* __restrict__ z, double* __restrict__ x) {
  const int s = item.s, i0 = item.r0, i1 = item.r1, w0 = item.w0;
  const int LG = 32 / WB;
  const int w = w0 + lane % WB;
  if (w >= W) return;
  const int rl = lane / WB;
  const int c0 = __ldg(F.col0 + s), k = __ldg(F.k + s), m = __ldg(F.m + s);
  const double* Fs = F.frow + __ldg(F.valptr + s);
  // contraction rows [c_lo, c_hi) of [i0, k + m): diagonal part r < k, off-diagonal part r >= k
  const int r_diag_end = min(k, item.c_hi);
  const int q_begin = max(item.c_lo, k) - k, q_end = max(item.c_hi, k) - k;
  double acc[kRowsPerLane];
  int ii[kRowsPerLane];
#pragma unroll
  for (int t = 0; t < kRowsPerLane; ++t) {
    acc[t] = 0.0;
    const int i = i0 + rl + t * LG;
    ii[t] = i < i1 ? i : i0;
  }
  // diagonal block: inv(L11)^T z_s (zero above the diagonal, so start at row i0)
  int r = max(i0, item.c_lo);
  for (; r + kUnroll <= r_diag_end; r += kUnroll) {
    double zr[kUnroll], fv[kUnroll][kRowsPerLane];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) zr[u] = __ldg(z + (int64_t)(c0 + r + u) * W + w);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int t = 0; t < kRowsPerLane; ++t) fv[u][t] = __ldg(Fs + (int64_t)(r + u) * k + ii[t]);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int t = 0; t < kRowsPerLane; ++t) acc[t] = fma(fv[u][t], zr[u], acc[t]);
  }
  for (; r < r_diag_end; ++r) {
    const double zr = __ldg(z + (int64_t)(c0 + r) * W + w);
    const double* row = Fs + (int64_t)r * k;
#pragma unroll
    for (int t = 0; t < kRowsPerLane; ++t) acc[t] = fma(__ldg(row + ii[t]), zr, acc[t]);
  }
  // off-diagonal rows: - (L21 inv(L11))^T x[R_s]; index loads, then value loads, then FMAs
  const int32_t* R = F.rows + __ldg(F.rowptr + s);
  int q = q_begin;
  for (; q + kUnroll <= q_end; q += kUnroll) {
    int idx[kUnroll];
    double xr[kUnroll], fv[kUnroll][kRowsPerLane];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) idx[u] = __ldg(R + q + u);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int t = 0; t < kRowsPerLane; ++t) fv[u][t] = __ldg(Fs + (int64_t)(k + q + u) * k + ii[t]);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) xr[u] = load_vec<kSharedLaunch>(x + (int64_t)idx[u] * W + w);
#pragma unroll
    for (int u = 0; u < kUnroll; ++u)
#pragma unroll
      for (int t = 0; t < kRowsPerLane; ++t) acc[t] = fma(-fv[u][t], xr[u], acc[t]);
  }
  for (; q < q_end; ++q) {
    const double xr = load_vec<kSharedLaunch>(x + (int64_t)__ldg(R + q) * W + w);
    const double* row = Fs + (int64_t)(k + q) * k;
#pragma unroll
    for (int t = 0; t < kRowsPerLane; ++t) acc[t] = fma(-__ldg(row + ii[t]), xr, acc[t]);
  }
#pragma unroll
  for (int t = 0; t < kRowsPerLane; ++t) {
    const int i = i0 + rl + t * LG;
    if (i >= i1) break;
    if (item.partial) atomicAdd(x + (int64_t)(c0 + i) * W + w, acc[t]);
    else x[(int64_t)(c0 + i) * W + w] = acc[t];
  }
  (void)m;
}

// level-synchronous sweeps: one launch per elimination-tree level, one warp per item (kPacks:
// the level also holds W = 1 packs; a separate instantiation keeps their registers out of the
// regular kernels)
template <int kRowsPerLane, bool kPacks>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_fwd_level(FactorDev F, const int4* __restrict__ items,
                                                                   int n_items, int W, int WB,
                                                                   double* __restrict__ b, double* __restrict__ z) {
  pdl_begin();
  const int it = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (it >= n_items) return;
  const int4 raw = items[it];
  if (kPacks && raw.x < 0) fwd_pack_any<false>(F, raw, threadIdx.x & 31, b, z);
  else fwd_item<kRowsPerLane, false>(F, unpack_item(raw), threadIdx.x & 31, W, WB, b, z);
}

template <int kRowsPerLane, bool kPacks>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_bwd_level(FactorDev F, const int4* __restrict__ items,
                                                                   int n_items, int W, int WB,
                                                                   const double* __restrict__ z, double* __restrict__ x) {
  pdl_begin();
  const int it = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (it >= n_items) return;
  const int4 raw = items[it];
  if (kPacks && raw.x < 0) bwd_pack_any<false>(F, raw, threadIdx.x & 31, z, x);
  else bwd_item<kRowsPerLane, false>(F, unpack_item(raw), threadIdx.x & 31, W, WB, z, x);
}

// ------------------------------------------------------------------------------------------
// Subtree sweeps (level schedule, 32 problems per warp). The bottom of the elimination tree is
// cut into subtrees of at most a few dozen rows: a subtree's columns are contiguous (postorder),
// every row outside it that a member touches is an off-diagonal row of its root (the structure
// of a column is contained in its parent's), so one warp can solve a whole subtree for its 32
// problems with the subtree's rows in shared memory: lane = problem, rows [0, ncols) are the
// subtree's columns, rows [ncols, ncols + m_root) the root's off-diagonal rows. Each lane walks
// the members in postorder (forward) or reverse postorder (backward) on its own column of that
// buffer, so no lane waits for another; the block's warps (consecutive 32-problem blocks of the
// same subtree) share the members' F values, staged once. This replaces the bottom levels'
// launches, their per-item index loads and the scatter atomics inside the subtree: one atomic per
// (outside row, problem) remains, and every row of b, z and x the subtree owns moves once.
// ------------------------------------------------------------------------------------------
struct SubTree {
  int s0, n;             // first member supernode, member count (the root is s0 + n - 1)
  int c0, ncols;         // first column, column count
  int m_root;            // the root's off-diagonal row count
  int f_len, l_len;      // the members' F values (row-major), entries of their local row maps
  int pad;
  int64_t f_off, l_off, r_off;   // into frow, the local row maps, and rows (the root's)
};

struct SubDev {
  const SubTree* tab = nullptr;
  const int4* meta = nullptr;      // per member supernode: column - c0, k, k + m, F offset - f_off
  const int32_t* lrow = nullptr;   // per member supernode: offset of its local row map - l_off
  const uint16_t* loc = nullptr;   // local row (in the subtree buffer) of every off-diagonal row
  int n = 0;                       // subtrees
  int max_rows = 0, max_f = 0, max_n = 0, max_l = 0;   // largest per subtree (max_f even)
};

// dynamic shared memory of a subtree launch with `warps` warps per block: the warps' row
// buffers, then F values, member metadata, local row map offsets and the local row maps
__host__ __device__ inline size_t sub_smem_bytes(const SubDev& S, int warps) {
  return (size_t)warps * S.max_rows * 32 * sizeof(double) + (size_t)S.max_f * sizeof(double) +
         (size_t)S.max_n * (sizeof(int4) + sizeof(int32_t)) + (size_t)S.max_l * sizeof(uint16_t);
}

// F value idx of a member: staged in shared memory (FS = 1) or interleaved by lane in global
// memory (FS = 32, the W = 1 subtree packs)
template <int FS>
__device__ __forceinline__ double sub_f(const double* Fr, int idx) {
  if (FS == 1) return Fr[idx];
  return __ldg(Fr + (int64_t)idx * FS);
}

// forward, one member with K columns: z rows from the buffer's b rows, then its off-diagonal
// rows updated in the buffer (b_R -= F21 b_s). `buf` points at this lane's row 0 (rows 32
// doubles apart), `zs` at z row c0 + c of this lane's problem.
template <int K, int FS = 1>
__device__ __forceinline__ void sub_fwd_member(const double* Fr, const uint16_t* L, int c, int nf, double* buf,
                                               double* zs, int64_t W) {
  double bs[K];
#pragma unroll
  for (int j = 0; j < K; ++j) bs[j] = buf[(c + j) * 32];
#pragma unroll
  for (int r = 0; r < K; ++r) {
    double acc = 0.0;
#pragma unroll
    for (int j = 0; j <= r; ++j) acc = fma(sub_f<FS>(Fr, r * K + j), bs[j], acc);
    zs[(int64_t)r * W] = acc;
  }
  // two rows at a time: a member's off-diagonal rows are distinct, so both loads go first
  int r = K;
  for (; r + 2 <= nf; r += 2) {
    const int l0 = L[r - K], l1 = L[r + 1 - K];
    double t0 = buf[l0 * 32], t1 = buf[l1 * 32];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      t0 = fma(-sub_f<FS>(Fr, r * K + j), bs[j], t0);
      t1 = fma(-sub_f<FS>(Fr, (r + 1) * K + j), bs[j], t1);
    }
    buf[l0 * 32] = t0;
    buf[l1 * 32] = t1;
  }
  if (r < nf) {
    const int l0 = L[r - K];
    double t0 = buf[l0 * 32];
#pragma unroll
    for (int j = 0; j < K; ++j) t0 = fma(-sub_f<FS>(Fr, r * K + j), bs[j], t0);
    buf[l0 * 32] = t0;
  }
}

// backward, one member: x_s = inv(L11)^T z_s - (L21 inv(L11))^T x_R with z_s in the buffer's
// own rows and x_R in its ancestors' rows (computed before, or loaded for the root's rows);
// x_s replaces z_s in the buffer and goes to x row c0 + c (`xs`)
template <int K, int FS = 1>
__device__ __forceinline__ void sub_bwd_member(const double* Fr, const uint16_t* L, int c, int nf, double* buf,
                                               double* xs, int64_t W) {
  double acc[K];
#pragma unroll
  for (int j = 0; j < K; ++j) acc[j] = 0.0;
#pragma unroll
  for (int r = 0; r < K; ++r) {
    const double zr = buf[(c + r) * 32];
#pragma unroll
    for (int j = 0; j <= r; ++j) acc[j] = fma(sub_f<FS>(Fr, r * K + j), zr, acc[j]);
  }
#pragma unroll 4
  for (int r = K; r < nf; ++r) {
    const double xr = buf[L[r - K] * 32];
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = fma(-sub_f<FS>(Fr, r * K + j), xr, acc[j]);
  }
#pragma unroll
  for (int j = 0; j < K; ++j) {
    buf[(c + j) * 32] = acc[j];
    xs[(int64_t)j * W] = acc[j];
  }
}

// one member of a subtree walk: the K-specialised walker of its width
template <bool kForward, int FS>
__device__ __forceinline__ void sub_member(int k, const double* Fr, const uint16_t* L, int c, int nf, double* buf,
                                           double* out, int64_t W) {
#define JJA_SUB_CASE(KK)                                                  \
  case KK:                                                                \
    if (kForward) sub_fwd_member<KK, FS>(Fr, L, c, nf, buf, out, W);     \
    else sub_bwd_member<KK, FS>(Fr, L, c, nf, buf, out, W);              \
    break;
  switch (k) {
    JJA_SUB_CASE(1)
    JJA_SUB_CASE(2)
    JJA_SUB_CASE(3)
    JJA_SUB_CASE(4)
    JJA_SUB_CASE(5)
    JJA_SUB_CASE(6)
    JJA_SUB_CASE(7)
    default:
      if (kForward) sub_fwd_member<8, FS>(Fr, L, c, nf, buf, out, W);
      else sub_bwd_member<8, FS>(Fr, L, c, nf, buf, out, W);
      break;
  }
#undef JJA_SUB_CASE
}

// grid (subtrees, ceil(problem blocks / warps per block)); block = warps per block x 32.
// Forward: b rows in, z rows out, the root's off-diagonal rows of b updated atomically.
// Backward: z rows and the root's off-diagonal rows of x in, x rows out.
template <bool kForward>
__global__ void __launch_bounds__(256) k_subtree(FactorDev F, SubDev S, int W, int w0, int wn,
                                                 double* __restrict__ b, double* __restrict__ z,
                                                 double* __restrict__ x) {
  pdl_begin();
  extern __shared__ double sub_sh[];
  const SubTree T = S.tab[blockIdx.x];
  const int nw = blockDim.x >> 5, wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* Fsh = sub_sh + (size_t)nw * S.max_rows * 32;
  int4* Msh = reinterpret_cast<int4*>(Fsh + S.max_f);
  int32_t* Lrow = reinterpret_cast<int32_t*>(Msh + S.max_n);
  uint16_t* Lsh = reinterpret_cast<uint16_t*>(Lrow + S.max_n);
  for (int i = threadIdx.x; i < T.f_len; i += blockDim.x) Fsh[i] = __ldg(F.frow + T.f_off + i);
  for (int i = threadIdx.x; i < T.n; i += blockDim.x) {
    Msh[i] = __ldg(S.meta + T.s0 + i);
    Lrow[i] = __ldg(S.lrow + T.s0 + i);
  }
  for (int i = threadIdx.x; i < T.l_len; i += blockDim.x) Lsh[i] = __ldg(S.loc + T.l_off + i);
  __syncthreads();
  const int w = w0 + (blockIdx.y * nw + wi) * 32 + lane;
  if (w >= w0 + wn || w >= W) return;
  double* buf = sub_sh + (size_t)wi * S.max_rows * 32 + lane;
  const int32_t* R = F.rows + T.r_off;
  const int64_t Wl = W;
  if (kForward) {
#pragma unroll 4
    for (int i = 0; i < T.ncols; ++i) buf[i * 32] = b[(int64_t)(T.c0 + i) * Wl + w];
    for (int q = 0; q < T.m_root; ++q) buf[(T.ncols + q) * 32] = 0.0;
    for (int i = 0; i < T.n; ++i) {
      const int4 mt = Msh[i];
      const double* Fr = Fsh + mt.w;
      const uint16_t* L = Lsh + Lrow[i];
      sub_member<true, 1>(mt.y, Fr, L, mt.x, mt.z, buf, z + (int64_t)(T.c0 + mt.x) * Wl + w, Wl);
    }
    for (int q = 0; q < T.m_root; ++q) atomicAdd(b + (int64_t)__ldg(R + q) * Wl + w, buf[(T.ncols + q) * 32]);
  } else {
#pragma unroll 4
    for (int q = 0; q < T.m_root; ++q) buf[(T.ncols + q) * 32] = __ldcg(x + (int64_t)__ldg(R + q) * Wl + w);
#pragma unroll 4
    for (int i = 0; i < T.ncols; ++i) buf[i * 32] = __ldg(z + (int64_t)(T.c0 + i) * Wl + w);
    for (int i = T.n - 1; i >= 0; --i) {
      const int4 mt = Msh[i];
      const double* Fr = Fsh + mt.w;
      const uint16_t* L = Lsh + Lrow[i];
      sub_member<false, 1>(mt.y, Fr, L, mt.x, mt.z, buf, x + (int64_t)(T.c0 + mt.x) * Wl + w, Wl);
    }
  }
}

// Subtree packs (below 32 problems per warp): subtrees of one shape (the same members, widths,
// heights and local row maps; the bottoms of lattices repeat a few hundred shapes) are grouped
// NS to a warp, NS = 32 / WB slots of WB lanes, one subtree per slot and one problem per lane,
// with their F values interleaved by slot (the load of a value index is NS contiguous doubles).
// Each lane walks its subtree for its problem as k_subtree's lanes do, on its own column of the
// warp's shared buffer; the shape's metadata and row maps are the same for every lane.
struct SubShape {
  int n, ncols, m_root, f_len;   // members, columns, root rows, F values per subtree
  int meta_off, pad;             // into meta and lrow (per member)
  int64_t loc_off;               // into loc
};

struct SubPackDev {
  const int4* items = nullptr;     // per warp: shape, slots | w0 << 6, first slot, F values offset / NS
  const SubShape* shapes = nullptr;
  const int4* meta = nullptr;      // per member of a shape: column, k, k + m, F offset (in the subtree)
  const int32_t* lrow = nullptr;   // per member of a shape: offset of its row map in the shape's loc
  const uint16_t* loc = nullptr;
  const int32_t* c0 = nullptr;     // per slot: the subtree's first column
  const int64_t* roff = nullptr;   // per slot: its root's rows in F.rows
  const double* vals = nullptr;    // F values, interleaved by slot
  int n_items = 0, max_rows = 0, ns = 0;   // ns: slots per warp (32 / problems per slot)
};

constexpr int kSubPackWarps = 4;   // warps per block (independent items)

template <bool kForward, int NS>
__global__ void __launch_bounds__(kSubPackWarps * 32) k_subtree_pack(FactorDev F, SubPackDev P, int W,
                                                                    double* __restrict__ b, double* __restrict__ z,
                                                                    double* __restrict__ x) {
  pdl_begin();
  extern __shared__ double subp_sh[];
  constexpr int WB = 32 / NS;
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int it = blockIdx.x * kSubPackWarps + wi;
  if (it >= P.n_items) return;
  const int4 item = P.items[it];
  const int slot = lane / WB, w = (item.y >> 6) + (lane - slot * WB);
  if (slot >= (item.y & 63) || w >= W) return;   // lanes walk independently: no synchronisation below
  const SubShape T = P.shapes[item.x];
  double* buf = subp_sh + (size_t)wi * P.max_rows * 32 + lane;
  const int64_t Wl = W;
  const int64_t c0 = __ldg(P.c0 + item.z + slot);
  const int32_t* R = F.rows + __ldg(P.roff + item.z + slot);
  const double* V = P.vals + (int64_t)item.w * NS + slot;
  const uint16_t* loc = P.loc + T.loc_off;
  if (kForward) {
#pragma unroll 4
    for (int i = 0; i < T.ncols; ++i) buf[i * 32] = b[(c0 + i) * Wl + w];
    for (int q = 0; q < T.m_root; ++q) buf[(T.ncols + q) * 32] = 0.0;
    for (int i = 0; i < T.n; ++i) {
      const int4 mt = __ldg(P.meta + T.meta_off + i);
      sub_member<true, NS>(mt.y, V + (int64_t)mt.w * NS, loc + __ldg(P.lrow + T.meta_off + i), mt.x, mt.z, buf,
                           z + (c0 + mt.x) * Wl + w, Wl);
    }
    for (int q = 0; q < T.m_root; ++q) atomicAdd(b + (int64_t)__ldg(R + q) * Wl + w, buf[(T.ncols + q) * 32]);
  } else {
#pragma unroll 4
    for (int q = 0; q < T.m_root; ++q) buf[(T.ncols + q) * 32] = __ldcg(x + (int64_t)__ldg(R + q) * Wl + w);
#pragma unroll 4
    for (int i = 0; i < T.ncols; ++i) buf[i * 32] = __ldg(z + (c0 + i) * Wl + w);
    for (int i = T.n - 1; i >= 0; --i) {
      const int4 mt = __ldg(P.meta + T.meta_off + i);
      sub_member<false, NS>(mt.y, V + (int64_t)mt.w * NS, loc + __ldg(P.lrow + T.meta_off + i), mt.x, mt.z, buf,
                            x + (c0 + mt.x) * Wl + w, Wl);
    }
  }
}

// the pack kernel of a slot count (32, 16, 8, 4 or 2 slots of 1, 2, 4, 8 or 16 problems)
using SubPackKernel = void (*)(FactorDev, SubPackDev, int, double*, double*, double*);
SubPackKernel sub_pack_kernel(bool forward, int ns) {
#define JJA_SUBP(N) \
  case N: return forward ? k_subtree_pack<true, N> : k_subtree_pack<false, N>;
  switch (ns) {
    JJA_SUBP(32)
    JJA_SUBP(16)
    JJA_SUBP(8)
    JJA_SUBP(4)
    JJA_SUBP(2)
    default: throw Error(JJA_ERR_INTERNAL, "subtree pack: bad slot count");
  }
#undef JJA_SUBP
}

// ------------------------------------------------------------------------------------------
// Dataflow sweeps: ONE launch per sweep. Warps take items in the sweep's topological order from
// a global counter; an item starts once the items it depends on have finished, which is
// tracked by per-supernode completion counters instead of a kernel boundary per level:
//   forward:  items of s wait until every item of s's children is done (children wait for
//             theirs, so the whole subtree, which scatters into b_s, is done);
//   backward: items of s wait until every item of s's parent is done (x of all ancestors).
// No deadlock: a warp only waits for items earlier in the order, and every such item was taken
// by a running warp before; the earliest unfinished item never waits. Every wait is bounded
// (kFlowSpinLimit polls); a wait that runs out records an error flag that the host reads
// (jja_plan_status), and the item then proceeds (its results are not to be used).
// ------------------------------------------------------------------------------------------
// polls of one wait (each a sleep of >= 64 ns plus an L2 round trip: 0.07-0.5 s in all), far
// beyond the longest level of any plan (~ms); after one wait has run out, all others give up at once
constexpr long long kFlowSpinLimit = 1LL << 20;

struct Flow {
  int* next;                    // item counter of this sweep (zeroed before the sweep)
  unsigned* done;               // per-supernode completed-item counters (zeroed before the sweep)
  const int32_t* wait_on;       // supernode whose counter an item of s waits on, or -1
  const uint32_t* wait_count;   // ... until it reaches this count
  const int32_t* notify;        // supernode whose counter an item of s increments when done, or -1
  int* err;                     // set to 1 when a wait ran out
};

__device__ __forceinline__ void flow_wait(const Flow& fl, int s) {
  const int t = __ldg(fl.wait_on + s);
  if (t < 0) return;
  const unsigned need = __ldg(fl.wait_count + s);
  const volatile unsigned* c = fl.done + t;
  const volatile int* err = fl.err;
  for (long long i = 0; *c < need; ++i) {
    if (i >= kFlowSpinLimit || *err) {
      atomicExch(fl.err, 1);
      return;
    }
    __nanosleep(64);
  }
  __threadfence();   // acquire: the producers' writes are visible before this item reads them
}

template <int kRowsPerLane, bool kForward>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) k_flow_sweep(FactorDev F, const int4* __restrict__ items,
                                                                    int n_items, int W, int WB, double* b,
                                                                    double* z, double* x, Flow fl) {
  pdl_begin();
  const int lane = threadIdx.x & 31;
  // the next item is taken while the current one runs (hides the counter's round trip); a
  // warp then holds two items, the later one not started, which keeps the order argument:
  // the earliest unfinished item is always the one its warp is working on
  int it = 0;
  if (lane == 0) it = atomicAdd(fl.next, 1);
  it = __shfl_sync(0xffffffffu, it, 0);
  while (it < n_items) {
    int nxt = 0;
    if (lane == 0) nxt = atomicAdd(fl.next, 1);
    const Item item = unpack_item(items[it]);
    if (lane == 0) flow_wait(fl, item.s);
    __syncwarp();
    if (kForward) fwd_item<kRowsPerLane, true>(F, item, lane, W, WB, b, z);
    else bwd_item<kRowsPerLane, true>(F, item, lane, W, WB, z, x);
    __syncwarp();      // the warp's results, then one release fence and the completion count
    if (lane == 0) {
      const int t = __ldg(fl.notify + item.s);
      if (t >= 0) {
        __threadfence();
        atomicAdd(fl.done + t, 1u);
      }
    }
    it = __shfl_sync(0xffffffffu, nxt, 0);
  }
}

// ------------------------------------------------------------------------------------------
// Cooperative sweeps (schedule 3): ONE launch per sweep that walks the elimination-tree levels
// itself, separated by a grid-wide barrier instead of a kernel boundary. Few problems per launch
// (a single array, a ragged union) leave the level kernels short and bound by their launch gaps
// (~5 us per level replayed from a graph); a barrier costs about a microsecond. The launch is
// cooperative, so all its blocks are resident at once and every block reaches every barrier.
// Face vectors written by earlier levels of the same launch are read through L2 (ld.global.cg).
// The barrier is a bounded spin: one that runs out sets the plan's error flag (jja_plan_check
// reports it) and lets the launch finish; once one has run out, the others give up at once.
// ------------------------------------------------------------------------------------------
constexpr int kCoopThreads = 512;                    // 16 warps per block, at most 2 blocks per SM:
constexpr int kCoopBlocksPerSM = 2;                  // few arrivals per barrier
constexpr long long kBarrierSpinLimit = 1LL << 22;   // polls of >= 32 ns: >= 0.13 s, far beyond any level

// the k-th barrier of a launch completes when the arrival counter (zero at the launch) reaches
// (k + 1) x gridDim.x; `target` is that count
__device__ __forceinline__ void grid_barrier(unsigned* count, unsigned target, int* err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();   // release: the block's writes (ordered by the CTA barrier) before the arrival
    atomicAdd(count, 1u);
    const volatile unsigned* c = count;
    const volatile int* e = err;
    for (long long i = 0; *c < target; ++i) {
      if (i >= kBarrierSpinLimit || *e) {
        atomicExch(err, 1);
        break;
      }
      __nanosleep(32);
    }
    __threadfence();   // acquire
  }
  __syncthreads();
}

// Phase 0 zeroes the rows that split dot products accumulate into (columns [w0, w0 + wn)) and
// the other sweep's barrier counter (sweeps alternate forward, backward on a stream, so each
// starts from a counter the previous one zeroed), then the levels run in order (forward: leaves
// first; backward: root first), every warp of the grid taking the level's items in turn.
template <int kRowsPerLane, bool kForward, bool kPacks>
__global__ void __launch_bounds__(kCoopThreads) k_coop_sweep(FactorDev F, const int4* __restrict__ items,
                                                             const int64_t* __restrict__ level_ptr, int n_levels,
                                                             int W, int WB, double* b, double* z, double* x,
                                                             const int32_t* __restrict__ zrows, int nz, int w0, int wn,
                                                             unsigned* bar, unsigned* other_bar, int* err,
                                                             unsigned unreachable) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, nth = (int64_t)gridDim.x * blockDim.x;
  double* acc = kForward ? z : x;
  for (int64_t e = tid; e < (int64_t)nz * wn; e += nth) {
    const int64_t i = e / wn, w = w0 + (e - i * wn);
    acc[(int64_t)__ldg(zrows + i) * W + w] = 0.0;
  }
  if (tid == 0) *other_bar = 0u;
  unsigned target = gridDim.x + unreachable;   // unreachable: 0, or 1 to test the barrier's bound
  grid_barrier(bar, target, err);
  const int64_t warp = tid >> 5, nwarps = nth >> 5;
  const int lane = threadIdx.x & 31;
  for (int q = 0; q < n_levels; ++q) {
    const int l = kForward ? q : n_levels - 1 - q;
    const int64_t i1 = __ldg(level_ptr + l + 1);
    for (int64_t it = __ldg(level_ptr + l) + warp; it < i1; it += nwarps) {
      const int4 raw = items[it];
      if (kForward) {
        if (kPacks && raw.x < 0) fwd_pack_any<true>(F, raw, lane, b, z);
        else fwd_item<kRowsPerLane, true>(F, unpack_item(raw), lane, W, WB, b, z);
      } else {
        if (kPacks && raw.x < 0) bwd_pack_any<true>(F, raw, lane, z, x);
        else bwd_item<kRowsPerLane, true>(F, unpack_item(raw), lane, W, WB, z, x);
      }
    }
    if (q + 1 < n_levels) {
      target += gridDim.x;
      grid_barrier(bar, target, err);
    }
  }
}

// ------------------------------------------------------------------------------------------
// Fast Poisson solve for uniform square arrays. With equal R, C and a uniform self-inductance l,
// K = kappa (4 I - adjacency) on the (mx x my) grid of faces, kappa = l + 1/(Cv + Rv): the
// 5-point Laplacian with Dirichlet boundaries, diagonalised by the sine transform (DST-I) along
// rows and columns, eigenvalues kappa (lx_kx + ly_ky), l_k = 2 - 2 cos(pi k / (m + 1)). A solve
// is three kernels and reads no factor: DST of every face row; per column DST, division by the
// eigenvalues (and the transforms' scale), inverse DST; inverse DST of every row. Each DST-I of
// length m = N - 1 is the imaginary part of a radix-2 FFT of the odd extension (length 2N, N a
// power of two) in shared memory: y_k = -Im(FFT(e))_k / 2, e = (0, x, 0, -reverse(x)).
// (A sparse supernodal solve of the same matrix is a chain of tree levels, each a few dependent
// memory round trips; three short launches beat it for few problems per launch.)
// ------------------------------------------------------------------------------------------
struct DstArgs {
  int mx, my;                  // faces per grid row, grid rows
  int lgx, lgy;                // log2 of the FFT lengths 2 (mx + 1), 2 (my + 1)
  const int32_t* grid_face;    // per cell iy * mx + ix: the face (factor's order)
  const double2* twx;          // exp(-2 pi i k / (2 (mx + 1))), k < mx + 1
  const double2* twy;
  const double* lamx;          // 2 - 2 cos(pi (k + 1) / (mx + 1)), k < mx
  const double* lamy;
  double scale;                // (2 / (mx + 1)) (2 / (my + 1)) / kappa
  double* t1;                  // scratch, (W, my, mx) problem-major
  double* t2;
};

// Two lines per transform: z = e1 + i e2 for the odd extensions e1, e2 of x1 and x2 (m values
// each at x[j * stride]; x2 may be null), loaded in bit-reversed order and transformed in place.
// As e1 and e2 are real, the DST-I of x1 is -(Im Z_k - Im Z_{n-k}) / 4 and that of x2 is
// (Re Z_k - Re Z_{n-k}) / 4, k = 1..m (dst_pair_out): half the butterflies of one FFT per line.
__device__ __forceinline__ void dst_pair(double2* a, const double* x1, const double* x2, int64_t stride, int m, int lg,
                                         const double2* tw) {
  const int n = 2 * (m + 1), N = m + 1;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double e1 = 0.0, e2 = 0.0;
    if (i >= 1 && i <= m) {
      e1 = x1[(int64_t)(i - 1) * stride];
      if (x2) e2 = x2[(int64_t)(i - 1) * stride];
    } else if (i > N) {
      e1 = -x1[(int64_t)(n - i - 1) * stride];
      if (x2) e2 = -x2[(int64_t)(n - i - 1) * stride];
    }
    a[__brev((unsigned)i) >> (32 - lg)] = make_double2(e1, e2);
  }
  __syncthreads();
  for (int l = 1; l <= lg; ++l) {
    const int half = 1 << (l - 1), tstride = n >> l;
    for (int j = threadIdx.x; j < n / 2; j += blockDim.x) {
      const int pos = j & (half - 1);
      const int i0 = ((j >> (l - 1)) << l) + pos, i1 = i0 + half;
      const double2 w = tw[pos * tstride];
      const double2 u = a[i0], v = a[i1];
      const double2 t = make_double2(fma(w.x, v.x, -w.y * v.y), fma(w.x, v.y, w.y * v.x));
      a[i0] = make_double2(u.x + t.x, u.y + t.y);
      a[i1] = make_double2(u.x - t.x, u.y - t.y);
    }
    __syncthreads();
  }
}

// One line per transform, at half the length: the odd extension e of x (n = 2N values, N = m + 1,
// real) packed as z_p = e_{2p} + i e_{2p+1}, p < N, loaded in bit-reversed order and transformed
// in place by an N-point FFT (twiddles W_N^q = W_n^{2q}); dst_line_out then forms the n-point
// transform of e from Z_k and Z_{N-k}. Half the butterflies of the n-point transform, one line
// per block (all SMs busy where pairing two lines would halve the blocks).
__device__ __forceinline__ void dst_line(double2* a, const double* x, int64_t stride, int m, int lg,
                                         const double2* tw) {
  const int N = m + 1, n = 2 * N, lgN = lg - 1;
  auto ext = [&](int j) -> double {   // e_j
    if (j >= 1 && j <= m) return x[(int64_t)(j - 1) * stride];
    if (j > N) return -x[(int64_t)(n - j - 1) * stride];
    return 0.0;
  };
  for (int p = threadIdx.x; p < N; p += blockDim.x)
    a[__brev((unsigned)p) >> (32 - lgN)] = make_double2(ext(2 * p), ext(2 * p + 1));
  __syncthreads();
  for (int l = 1; l <= lgN; ++l) {
    const int half = 1 << (l - 1), tstride = (N >> l) * 2;
    for (int j = threadIdx.x; j < N / 2; j += blockDim.x) {
      const int pos = j & (half - 1);
      const int i0 = ((j >> (l - 1)) << l) + pos, i1 = i0 + half;
      const double2 w = tw[pos * tstride];
      const double2 u = a[i0], v = a[i1];
      const double2 t = make_double2(fma(w.x, v.x, -w.y * v.y), fma(w.x, v.y, w.y * v.x));
      a[i0] = make_double2(u.x + t.x, u.y + t.y);
      a[i1] = make_double2(u.x - t.x, u.y - t.y);
    }
    __syncthreads();
  }
}

// the line's DST-I value at k = 1..m: with A = Z_k, B = conj Z_{N-k}, the n-point transform is
// E_k = (A + B) / 2 - (i / 2) W_n^k (A - B), and the DST-I sum is -Im(E_k) / 2
__device__ __forceinline__ double dst_line_out(const double2* a, int N, int k, const double2* tw) {
  const double2 A = a[k], Bc = a[N - k], w = tw[k];
  const double re = fma(w.x, A.x - Bc.x, -w.y * (A.y + Bc.y));   // Re(W^k (A - B))
  return 0.25 * (re - (A.y - Bc.y));
}

// the twiddles of a transform into shared memory (visible after the caller's next barrier)
__device__ __forceinline__ void load_twiddles(double2* dst, const double2* __restrict__ src, int count) {
  for (int i = threadIdx.x; i < count; i += blockDim.x) dst[i] = __ldg(src + i);
}

// the two lines' DST-I values at k = 1..m from the transformed buffer
__device__ __forceinline__ double2 dst_pair_out(const double2* a, int n, int k) {
  const double2 zk = a[k], zn = a[n - k];
  return make_double2(-0.25 * (zk.y - zn.y), 0.25 * (zk.x - zn.x));
}

// rows: out(w, iy, k) = DST_x of rows iy = lines blockIdx.x .. + lines - 1 (lines: 1 or 2) of
// problem w0 + blockIdx.y; `in_faces`: the input is a face vector (N x W, factor's face order)
// read through grid_face, else a (W, my, mx) scratch; `out_faces` likewise for the output
__global__ void k_dst_rows(DstArgs d, const double* in, double* out, int W, int w0, int in_faces, int out_faces,
                           int lines) {
  extern __shared__ double2 fft_buf[];
  const int iy0 = lines * blockIdx.x, iy1 = iy0 + 1, w = w0 + blockIdx.y, n = 2 * (d.mx + 1);
  const bool two = lines == 2 && iy1 < d.my;
  double2* tws = fft_buf + n + d.mx;   // after the FFT buffer and two lines (2 mx doubles)
  load_twiddles(tws, d.twx, n / 2);
  const double *src0, *src1 = nullptr;
  if (in_faces) {
    // gather both rows through the face map after the FFT buffer
    double* rows = reinterpret_cast<double*>(fft_buf + n);
    for (int j = threadIdx.x; j < d.mx; j += blockDim.x) {
      rows[j] = in[(int64_t)__ldg(d.grid_face + iy0 * d.mx + j) * W + w];
      if (two) rows[d.mx + j] = in[(int64_t)__ldg(d.grid_face + iy1 * d.mx + j) * W + w];
    }
    __syncthreads();
    src0 = rows;
    if (two) src1 = rows + d.mx;
  } else {
    src0 = in + ((int64_t)w * d.my + iy0) * d.mx;
    if (two) src1 = src0 + d.mx;
  }
  if (two) dst_pair(fft_buf, src0, src1, 1, d.mx, d.lgx, tws);
  else dst_line(fft_buf, src0, 1, d.mx, d.lgx, tws);
  for (int k = threadIdx.x; k < d.mx; k += blockDim.x) {
    const double2 y = two ? dst_pair_out(fft_buf, n, k + 1)
                          : make_double2(dst_line_out(fft_buf, d.mx + 1, k + 1, tws), 0.0);
    if (out_faces) {
      out[(int64_t)__ldg(d.grid_face + iy0 * d.mx + k) * W + w] = y.x;
      if (two) out[(int64_t)__ldg(d.grid_face + iy1 * d.mx + k) * W + w] = y.y;
    } else {
      out[((int64_t)w * d.my + iy0) * d.mx + k] = y.x;
      if (two) out[((int64_t)w * d.my + iy1) * d.mx + k] = y.y;
    }
  }
}

// columns kx = lines blockIdx.x .. + lines - 1: DST_y, division by the eigenvalues times the
// scale, inverse DST_y (DST-I is its own inverse up to the scale)
__global__ void k_dst_cols(DstArgs d, int w0, int lines) {
  extern __shared__ double2 fft_buf[];
  const int kx0 = lines * blockIdx.x, kx1 = kx0 + 1, w = w0 + blockIdx.y, n = 2 * (d.my + 1);
  const bool two = lines == 2 && kx1 < d.mx;
  const double* col = d.t1 + (int64_t)w * d.my * d.mx + kx0;
  double* tmp = reinterpret_cast<double*>(fft_buf + n);   // 2 x my values after the FFT buffer
  double2* tws = fft_buf + n + d.my;                      // then the twiddles
  load_twiddles(tws, d.twy, n / 2);
  if (two) dst_pair(fft_buf, col, col + 1, d.mx, d.my, d.lgy, tws);
  else dst_line(fft_buf, col, d.mx, d.my, d.lgy, tws);
  const double lx0 = __ldg(d.lamx + kx0), lx1 = two ? __ldg(d.lamx + kx1) : 0.0;
  for (int k = threadIdx.x; k < d.my; k += blockDim.x) {
    const double2 y = two ? dst_pair_out(fft_buf, n, k + 1)
                          : make_double2(dst_line_out(fft_buf, d.my + 1, k + 1, tws), 0.0);
    const double ly = __ldg(d.lamy + k);
    tmp[k] = y.x * d.scale / (lx0 + ly);
    tmp[d.my + k] = two ? y.y * d.scale / (lx1 + ly) : 0.0;
  }
  __syncthreads();
  if (two) dst_pair(fft_buf, tmp, tmp + d.my, 1, d.my, d.lgy, tws);
  else dst_line(fft_buf, tmp, 1, d.my, d.lgy, tws);
  double* out = d.t2 + (int64_t)w * d.my * d.mx + kx0;
  for (int k = threadIdx.x; k < d.my; k += blockDim.x) {
    const double2 y = two ? dst_pair_out(fft_buf, n, k + 1)
                          : make_double2(dst_line_out(fft_buf, d.my + 1, k + 1, tws), 0.0);
    out[(int64_t)k * d.mx] = y.x;
    if (two) out[(int64_t)k * d.mx + 1] = y.y;
  }
}

// ------------------------------------------------------------------------------------------
// Adjoint (backward through time) of the width-3 step theta_n = Q x_n + const, with
// x_n = Ic sin(phi_n) + c1 th_{n-1} + c2 th_{n-2} - Is, phi_n = 2 th_{n-1} - th_{n-2},
// Q = D A^T K^-1 A D - D, D = diag(1/c0) (symmetric, so Q^T = Q and one factor serves).
// With a_n = dL/dtheta_n and mu_n = Q a_n:
//   a_n = G_n + (2 Ic cos phi_{n+1} + c1) mu_{n+1} + (-Ic cos phi_{n+2} + c2) mu_{n+2}
//   dL/dIc += mu_n sin phi_n,  dL/dIs = -sum mu_n,  dL/df = -2 pi K^-1 A D sum a_n.
// A step is: k_adj_a (a_n -> u = D a_n), the face kernel (b = A u), the two triangular
// sweeps (nu = K^-1 b), k_adj_mu (mu_n = D A^T nu - u, sin/cos phi_n, accumulations).
// ------------------------------------------------------------------------------------------
struct AdjArgs {
  int Nj, W;
  jja_view G;
  const double* th_m1;
  const double* th_m2;
  const double* mu_p1;
  const double* mu_p2;
  const double* cos_p1;
  const double* cos_p2;
  double* mu_out;
  double* cos_out;
  double* usum;
  double* musum;
  double* gIc;
};

__global__ void __launch_bounds__(256) k_adj_a(AdjArgs a, Tables t, double* __restrict__ u) {
  const int64_t NjW = (int64_t)a.Nj * a.W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < NjW; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / a.W, w = e - j * a.W;
    double v = view_at(a.G, j, w);
    const double ic = __ldg(t.Ic + (t.ic_per_w ? e : j));
    if (a.mu_p1) v = fma(fma(2.0 * ic, a.cos_p1[e], __ldg(t.coef + j)), a.mu_p1[e], v);
    if (a.mu_p2) v = fma(fma(-ic, a.cos_p2[e], __ldg(t.coef + a.Nj + j)), a.mu_p2[e], v);
    const double uu = v * __ldg(t.inv_c0 + j);
    u[e] = uu;
    a.usum[e] += uu;
  }
}

__global__ void __launch_bounds__(256) k_adj_mu(AdjArgs a, Tables t, const double* __restrict__ u,
                                                const double* __restrict__ nu) {
  const int64_t NjW = (int64_t)a.Nj * a.W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < NjW; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / a.W, w = e - j * a.W;
    const int p0 = __ldg(t.jf_face + 2 * j), p1 = __ldg(t.jf_face + 2 * j + 1);
    double y = p0 >= 0 ? signed_by(nu[(int64_t)(p0 >> 1) * a.W + w], p0 & 1) : 0.0;
    if (p1 >= 0) y += signed_by(nu[(int64_t)(p1 >> 1) * a.W + w], p1 & 1);
    const double mu = fma(y, __ldg(t.inv_c0 + j), -u[e]);
    double s, c;
    fast_sincos(fma(2.0, a.th_m1[e], -a.th_m2[e]), t.sincos, s, c);
    a.mu_out[e] = mu;
    a.cos_out[e] = c;
    a.gIc[e] = fma(mu, s, a.gIc[e]);
    a.musum[e] += mu;
  }
}

// Vortex configurations n_s(f, w) = -sum_j A_fj round(theta_s(j, w) / 2 pi) of n_steps stored
// phase arrays (time_evolution.py:734-755; np.round is round-half-even, as rint), written in
// the original face order when n_out is given, and the vortex flow per problem,
// flow[w] += sum_f sum_{s >= 1} |n_s - n_{s-1}| (the numerator of AnnealingProblem's vortex
// mobility, time_evolution.py:1131-1136), when flow is given. One thread per (face, problem).
__global__ void __launch_bounds__(256) k_vortex(const double* __restrict__ theta, int64_t n_steps, int Nj, int Nf,
                                                int W, Tables t, int32_t* __restrict__ n_out,
                                                unsigned long long* __restrict__ flow) {
  const int64_t NfW = (int64_t)Nf * W, NjW = (int64_t)Nj * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < NfW; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = e / W, w = e - p * W;
    const int64_t i0 = __ldg(t.fj_ptr + p), i1 = __ldg(t.fj_ptr + p + 1);
    const int64_t fo = __ldg(t.face_orig + p);
    long long prev = 0, moved = 0;
    for (int64_t s = 0; s < n_steps; ++s) {
      const double* th = theta + s * NjW;
      long long n = 0;
      for (int64_t i = i0; i < i1; ++i) {
        const int code = __ldg(t.fj_col + i);          // (junction << 1) | (A entry is -1)
        const long long r = (long long)rint(th[(int64_t)(code >> 1) * W + w] / kTwoPi);
        n += (code & 1) ? r : -r;                      // n = -A round(theta / 2 pi)
      }
      if (n_out) n_out[s * NfW + fo * W + w] = (int32_t)n;
      if (s > 0) moved += n > prev ? n - prev : prev - n;
      prev = n;
    }
    if (flow && moved) atomicAdd(flow + w, (unsigned long long)moved);
  }
}

__global__ void k_unpermute_scaled(const double* __restrict__ src, double* __restrict__ dst,
                                   const int32_t* __restrict__ perm, int n, int W, double scale) {
  const int64_t nW = (int64_t)n * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nW; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / W, w = e - i * W;
    dst[(int64_t)__ldg(perm + i) * W + w] = scale * src[e];
  }
}

__global__ void k_eval_sin(const double* __restrict__ x, double* __restrict__ out, int64_t n,
                           const longlong2* __restrict__ tab) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = fast_sin(x[i], tab);
}

__global__ void k_permute_rows(const double* __restrict__ src, double* __restrict__ dst, const int32_t* __restrict__ map,
                               int n, int W, int gather) {
  const int64_t nW = (int64_t)n * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nW; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / W, w = e - i * W;
    const int64_t o = __ldg(map + i);
    if (gather) dst[e] = src[o * W + w];
    else dst[o * W + w] = src[e];
  }
}

int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, 152LL * 32));
}

template <class T>
T* upload(const T* h, size_t n, int64_t& bytes) {
  T* d = nullptr;
  const size_t alloc = n ? n : 1;
  JJA_CUDA(cudaMalloc(&d, alloc * sizeof(T)));
  bytes += (int64_t)(alloc * sizeof(T));
  if (h && n) JJA_CUDA(cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice));
  return d;
}

// rows per lane of the forward or backward sweep: rows_per_lane_fwd (forward only) overrides
// rows_per_lane, which sets both; unset fields take each sweep's default. Measured on GB300
// (ms/step, forward/backward rows): W = 512: 1/1 1.554, 2/1 1.511, 2/2 1.579; W = 1: 1/1 0.133,
// 2/1 0.138; 64x64 x 64: 1/1 0.138, 2/1 0.141; so two forward rows from W = 256 on.
// rows per lane of a sweep's work items for W problems on n faces (the forward sweep takes two
// from W = 256 on, and from W = 8 on arrays of 2^17 faces or more; measured on GB300:
// SquareArray(512,512) x 8 0.679 -> 0.663 ms, (1024,1024) x 8 2.43 -> 2.32 ms per step,
// (256,256) x 8 0.252 -> 0.267 ms)
int rows_per_lane_of(const jja_solve_tuning& tu, bool forward, int W, int n) {
  if (forward && tu.rows_per_lane_fwd) return tu.rows_per_lane_fwd;
  if (tu.rows_per_lane) return tu.rows_per_lane;
  if (forward && (W >= 256 || (W >= 8 && n >= kFwdWideFaces))) return kDefaultRowsPerLaneFwdWide;
  return kDefaultRowsPerLane;
}

// dot products of levels with fewer work items than this are split (split target): wider for
// 2-16 problems (measured on GB300: SquareArray(1024,1024) x 8 2.56 -> 2.43 ms per step,
// (512,512) x 8 0.699 -> 0.679; unchanged at W = 1 and W = 512 on 128x128 and 512x512)
int target_warps_of(const jja_solve_tuning& tu, int W) {
  if (tu.target_warps) return tu.target_warps;
  return (W >= 2 && W <= 16) ? kDefaultTargetWarpsSmallW : kDefaultTargetWarps;
}

// problems per warp of the triangular solves
int resolve_rhs_block(int W, const jja_solve_tuning& tu) {
  int WB = 1;
  while (WB < std::min(W, 32)) WB <<= 1;
  if (tu.rhs_block) {
    if (tu.rhs_block < 1 || tu.rhs_block > 32 || (tu.rhs_block & (tu.rhs_block - 1)))
      throw Error(JJA_ERR_ARG, "rhs_block must be a power of two <= 32");
    WB = tu.rhs_block;
  }
  return WB;
}

// Work items of both sweeps and the dataflow dependencies, built on the host.
struct Schedule {
  int n_levels = 0, ns = 0;
  std::vector<int4> fi;        // forward items, levels ascending (leaves first)
  std::vector<int4> bi;        // backward items, levels ascending (level launches run them per level, root first)
  std::vector<int4> bi_flow;   // the backward items root first (the dataflow sweep takes them in this order)
  std::vector<int64_t> fwd_ptr, bwd_ptr;   // per level, into fi / bi
  std::vector<char> level_packed;          // per level: holds W = 1 packs
  std::vector<int32_t> zf, zb;             // rows of z / x that partial items accumulate into
  // forward: items of s wait until done[fon[s]] == fcnt[s] (fon[s] = s or -1) and then count
  // towards fnot[s] (the parent); backward: items of s wait until done[bon[s]] == bcnt[s]
  // (bon[s] = parent or -1) and count towards bnot[s] (s itself, if it has children)
  std::vector<int32_t> fon, fnot, bon, bnot;
  std::vector<uint32_t> fcnt, bcnt;
  // W = 1 packs (level schedule only): 32 lanes each, the supernode of every lane (-1: none),
  // its (col0, k, k + m, rowptr) and the interleaved values (see fwd_pack)
  std::vector<int32_t> pack_sn;
  std::vector<int4> pack_meta;
  std::vector<double> pack_vals;
  // subtree sweeps (k_subtree): the subtrees, per supernode metadata (members only), the local
  // row maps, the largest subtree's sizes; their members have no level items
  std::vector<SubTree> subs;
  std::vector<int4> sub_meta;
  std::vector<int32_t> sub_lrow;
  std::vector<uint16_t> sub_loc;
  int sub_max_rows = 0, sub_max_f = 0, sub_max_n = 0, sub_max_l = 0;
  int sub_total = 0, sub_members = 0, sub_rows_max = 0;   // kept when the tables become packs
  // below 32 problems per warp: the subtrees grouped by shape into warps (k_subtree_pack; the
  // tables above are then empty)
  std::vector<int4> sp_items, sp_meta;
  std::vector<SubShape> sp_shapes;
  std::vector<int32_t> sp_lrow, sp_c0;
  std::vector<uint16_t> sp_loc;
  std::vector<int64_t> sp_roff;
  std::vector<double> sp_vals;
  int sp_max_rows = 0, sp_ns = 0;
};

// the supernodes a work item covers: one, or the members of a W = 1 pack
template <class Fn>
void for_each_supernode(const Schedule& S, const int4& v, Fn fn) {
  if (v.x >= 0) {
    fn(v.x);
    return;
  }
  const int64_t first = (-1 - (int64_t)v.x) * 32;
  if (v.y < 1 || v.y > 32 || first + 32 > (int64_t)S.pack_sn.size()) throw Error(JJA_ERR_INTERNAL, "pack out of range");
  for (int l = 0; l < v.y; ++l) fn(S.pack_sn[first + l]);
}

// Subtrees for k_subtree: the largest subtrees whose columns plus their root's off-diagonal rows
// number at most `max_rows`, with no member wider than kSubMaxK columns and bounded staging (F
// values, local row maps). Every limit grows towards the root, so a qualifying supernode's
// descendants qualify and the subtrees are the qualifying supernodes whose parent does not.
// Marks the members in `inside`, re-levels the others in `level` (leaves 0, all subtrees below
// level 0) and sets S.n_levels.
void build_subtrees(const jja::Factor& F, int max_rows, Schedule& S, std::vector<char>& inside,
                    std::vector<int>& level) {
  const int ns = F.ns;
  std::vector<int64_t> cols(ns), fl(ns), ll(ns);
  std::vector<int> kmax(ns), cnt(ns);
  for (int s = 0; s < ns; ++s) {
    const int k = F.sn_k[s], m = F.sn_m[s];
    cols[s] = k;
    fl[s] = (int64_t)(k + m) * k;
    ll[s] = m;
    kmax[s] = k;
    cnt[s] = 1;
  }
  for (int s = 0; s < ns; ++s) {
    const int p = F.sn_parent[s];
    if (p < 0) continue;
    if (p <= s || p >= ns) throw Error(JJA_ERR_INTERNAL, "supernodes are not in postorder");
    cols[p] += cols[s];
    fl[p] += fl[s];
    ll[p] += ll[s];
    kmax[p] = std::max(kmax[p], kmax[s]);
    cnt[p] += cnt[s];
  }
  std::vector<char> ok(ns);
  for (int s = 0; s < ns; ++s)
    ok[s] = cols[s] + F.sn_m[s] <= max_rows && kmax[s] <= kSubMaxK && fl[s] <= kSubMaxF && ll[s] <= kSubMaxL;
  S.sub_meta.assign(ns, make_int4(0, 0, 0, 0));
  S.sub_lrow.assign(ns, 0);
  for (int t = 0; t < ns; ++t) {
    const int p = F.sn_parent[t];
    if (!ok[t] || (p >= 0 && ok[p])) continue;
    SubTree T{};
    T.n = cnt[t];
    T.s0 = t - cnt[t] + 1;
    T.c0 = F.sn_col0[T.s0];
    T.ncols = (int)cols[t];
    T.m_root = F.sn_m[t];
    if (T.c0 + T.ncols != F.sn_col0[t] + F.sn_k[t]) throw Error(JJA_ERR_INTERNAL, "subtree columns are not contiguous");
    T.f_off = F.sn_valptr[T.s0];
    T.f_len = (int)(F.sn_valptr[t + 1] - T.f_off);
    T.r_off = F.sn_rowptr[t];
    T.l_off = (int64_t)S.sub_loc.size();
    T.l_len = (int)(F.sn_rowptr[t + 1] - F.sn_rowptr[T.s0]);
    const int c_end = T.c0 + T.ncols;
    const int* Rr = F.rows.data() + F.sn_rowptr[t];
    for (int u = T.s0; u <= t; ++u) {
      if (!ok[u] || inside[u]) throw Error(JJA_ERR_INTERNAL, "subtree member does not qualify");
      inside[u] = 1;
      const int k = F.sn_k[u];
      S.sub_meta[u] = make_int4(F.sn_col0[u] - T.c0, k, k + F.sn_m[u], (int)(F.sn_valptr[u] - T.f_off));
      S.sub_lrow[u] = (int32_t)(F.sn_rowptr[u] - F.sn_rowptr[T.s0]);
      for (int64_t q = F.sn_rowptr[u]; q < F.sn_rowptr[u + 1]; ++q) {
        const int r = F.rows[q];
        int local;
        if (r >= T.c0 && r < c_end) {
          local = r - T.c0;
        } else {
          const int* hit = std::lower_bound(Rr, Rr + T.m_root, r);
          if (hit == Rr + T.m_root || *hit != r) throw Error(JJA_ERR_INTERNAL, "subtree row outside its root's structure");
          local = T.ncols + (int)(hit - Rr);
        }
        S.sub_loc.push_back((uint16_t)local);
      }
    }
    S.sub_max_rows = std::max(S.sub_max_rows, T.ncols + T.m_root);
    S.sub_rows_max = S.sub_max_rows;
    S.sub_members += T.n;
    S.sub_max_f = std::max(S.sub_max_f, (T.f_len + 1) / 2 * 2);
    S.sub_max_n = std::max(S.sub_max_n, T.n);
    S.sub_max_l = std::max(S.sub_max_l, T.l_len);
    S.subs.push_back(T);
  }
  S.sub_total = (int)S.subs.size();
  // the remaining supernodes: leaves (or parents of subtrees only) at level 0
  int top = -1;
  for (int s = 0; s < ns; ++s) if (!inside[s]) level[s] = 0;
  for (int s = 0; s < ns; ++s) {
    if (inside[s]) continue;
    top = std::max(top, level[s]);
    const int p = F.sn_parent[s];
    if (p >= 0) level[p] = std::max(level[p], level[s] + 1);
  }
  S.n_levels = top + 1;
}

// Below 32 problems per warp: the subtrees of S (build_subtrees) grouped NS = 32 / WB to a warp by
// shape: equal member count, columns, root rows, per-member (column, k, k + m, F offset, row-map
// offset) and row maps, so a warp's lanes run the same walk; their F values (row-major per
// member) interleaved by slot; one item per pack and block of WB problems in [w_lo, w_hi).
// Replaces S's per-subtree tables.
void build_subtree_packs(const jja::Factor& F, Schedule& S, int WB, int w_lo, int w_hi) {
  const int NS = 32 / WB;
  std::map<std::vector<int>, std::vector<int>> by_shape;
  for (int t = 0; t < (int)S.subs.size(); ++t) {
    const SubTree& T = S.subs[t];
    std::vector<int> sig = {T.n, T.ncols, T.m_root, T.f_len, T.l_len};
    for (int u = T.s0; u < T.s0 + T.n; ++u) {
      const int4 mt = S.sub_meta[u];
      sig.insert(sig.end(), {mt.x, mt.y, mt.z, mt.w, S.sub_lrow[u]});
    }
    for (int64_t q = 0; q < T.l_len; ++q) sig.push_back(S.sub_loc[T.l_off + q]);
    by_shape[sig].push_back(t);
  }
  for (const auto& kv : by_shape) {
    const std::vector<int>& ts = kv.second;
    const SubTree& T0 = S.subs[ts[0]];
    SubShape sh{};
    sh.n = T0.n;
    sh.ncols = T0.ncols;
    sh.m_root = T0.m_root;
    sh.f_len = T0.f_len;
    sh.meta_off = (int)S.sp_meta.size();
    sh.loc_off = (int64_t)S.sp_loc.size();
    for (int u = T0.s0; u < T0.s0 + T0.n; ++u) {
      S.sp_meta.push_back(S.sub_meta[u]);
      S.sp_lrow.push_back(S.sub_lrow[u]);
    }
    S.sp_loc.insert(S.sp_loc.end(), S.sub_loc.begin() + T0.l_off, S.sub_loc.begin() + T0.l_off + T0.l_len);
    const int shape = (int)S.sp_shapes.size();
    S.sp_shapes.push_back(sh);
    S.sp_max_rows = std::max(S.sp_max_rows, sh.ncols + sh.m_root);
    for (size_t i = 0; i < ts.size(); i += NS) {
      const int count = (int)std::min<size_t>(NS, ts.size() - i);
      const int64_t lane0 = (int64_t)S.sp_c0.size(), off = (int64_t)S.sp_vals.size() / NS;
      if (lane0 >= INT32_MAX || off >= INT32_MAX) throw Error(JJA_ERR_ARG, "too many subtree packs");
      S.sp_vals.resize(S.sp_vals.size() + (size_t)NS * sh.f_len, 0.0);
      double* vals = S.sp_vals.data() + off * NS;
      for (int l = 0; l < NS; ++l) {
        if (l >= count) {
          S.sp_c0.push_back(0);
          S.sp_roff.push_back(0);
          continue;
        }
        const SubTree& T = S.subs[ts[i + l]];
        S.sp_c0.push_back(T.c0);
        S.sp_roff.push_back(T.r_off);
        // F row-major per member, at the member's offset in the subtree
        for (int u = T.s0; u < T.s0 + T.n; ++u) {
          const int k = F.sn_k[u], nf = k + F.sn_m[u];
          const double* src = F.fcol.data() + F.sn_valptr[u];
          const int64_t f = F.sn_valptr[u] - T.f_off;
          for (int r = 0; r < nf; ++r)
            for (int j = 0; j < k; ++j) vals[(f + (int64_t)r * k + j) * NS + l] = src[(int64_t)j * nf + r];
        }
      }
      for (int w0 = w_lo; w0 < w_hi; w0 += WB) {
        if (w0 >= (1 << 25)) throw Error(JJA_ERR_ARG, "subtree packs: too many problems");
        S.sp_items.push_back(make_int4(shape, count | (w0 << 6), (int)lane0, (int)off));
      }
    }
  }
  S.sp_ns = NS;
  S.subs.clear();
  S.sub_meta.clear();
  S.sub_lrow.clear();
  S.sub_loc.clear();
  S.sub_max_rows = S.sub_max_f = S.sub_max_n = S.sub_max_l = 0;
}

// the work items of problems [w_lo, w_hi) (w_hi < 0: all W); w_lo a multiple of the RHS block
Schedule build_schedule(const jja::Factor& F, int W, const jja_solve_tuning& tu, int w_lo = 0, int w_hi = -1) {
  if (W <= 0 || W >= (1 << 30)) throw Error(JJA_ERR_ARG, "W must be in [1, 2^30)");
  for (int v : {tu.rows_per_lane, tu.rows_per_lane_fwd})
    if (v && v != 1 && v != 2 && v != 4 && v != 8)
      throw Error(JJA_ERR_ARG, "rows_per_lane and rows_per_lane_fwd must be 1, 2, 4 or 8");
  if (tu.target_warps < 0 || tu.min_piece < 0) throw Error(JJA_ERR_ARG, "target_warps and min_piece must be >= 0");
  if (tu.schedule < 0 || tu.schedule > 3) throw Error(JJA_ERR_ARG, "schedule must be 0, 1, 2 or 3");
  if (tu.coop_blocks < 0) throw Error(JJA_ERR_ARG, "coop_blocks must be >= 0");
  if (tu.dst_lines < 0 || tu.dst_lines > 2) throw Error(JJA_ERR_ARG, "dst_lines must be 0, 1 or 2");
  if (tu.subtree_rows > kSubMaxRows) throw Error(JJA_ERR_ARG, "subtree_rows must be <= 64");
  if (tu.pdl < 0 || tu.pdl > 1) throw Error(JJA_ERR_ARG, "pdl must be 0 or 1");
  if (tu.pack_rows > 256) throw Error(JJA_ERR_ARG, "pack_rows must be <= 256");
  if (tu.pack_min_warps < 0) throw Error(JJA_ERR_ARG, "pack_min_warps must be >= 0");
  if (tu.pack_lanes != 0 && tu.pack_lanes != 1 && tu.pack_lanes != 2 && tu.pack_lanes != 4)
    throw Error(JJA_ERR_ARG, "pack_lanes must be 0, 1, 2 or 4");
  if (tu.groups < 0 || tu.groups > 64) throw Error(JJA_ERR_ARG, "groups must be in [0, 64]");
  const int WB = resolve_rhs_block(W, tu);
  if (w_hi < 0) w_hi = W;
  if (w_lo < 0 || w_lo >= w_hi || w_hi > W || w_lo % WB) throw Error(JJA_ERR_INTERNAL, "bad problem range");
  // W = 1 packs of small supernodes (level schedule only: the dataflow sweep counts items per
  // supernode)
  const int pack_rows = (W == 1 && tu.schedule != 2 && tu.pack_rows >= 0)
                            ? (tu.pack_rows ? tu.pack_rows : kDefaultPackRows) : 0;

  const int64_t pack_min_warps = tu.pack_min_warps ? tu.pack_min_warps : kDefaultPackMinWarps;
  const int target_warps = target_warps_of(tu, W);
  const int min_piece = tu.min_piece ? tu.min_piece : kDefaultMinPiece;
  const int LG = 32 / WB;
  const int RPI_f = LG * rows_per_lane_of(tu, true, W, F.n), RPI_b = LG * rows_per_lane_of(tu, false, W, F.n);
  Schedule S;
  S.n_levels = F.n_levels;
  S.ns = F.ns;
  for (int s = 0; s < F.ns; ++s) {
    if (F.sn_level[s] < 0 || F.sn_level[s] >= F.n_levels) throw Error(JJA_ERR_INTERNAL, "supernode level out of range");
    if (F.sn_k[s] + F.sn_m[s] >= 65536) throw Error(JJA_ERR_ARG, "supernode with >= 65536 rows");
  }
  // subtree sweeps at the bottom of the tree (level schedule, 32 problems per warp); the other
  // supernodes are re-levelled above them
  const int sub_rows = (tu.schedule <= 1 && tu.subtree_rows >= 0)
                           ? (tu.subtree_rows ? tu.subtree_rows : (W == 1 ? kDefaultSubRows1 : kDefaultSubRows)) : 0;
  std::vector<int> level(F.sn_level.begin(), F.sn_level.end());
  std::vector<char> inside(F.ns, 0);
  if (sub_rows > 0) {
    build_subtrees(F, sub_rows, S, inside, level);
    // by default only where the subtree launch has warps enough to hide each warp's walk (a
    // subtree is walked member by member; the levels it replaces run its rows in parallel)
    if (WB == 32 && !tu.subtree_rows && (int64_t)S.subs.size() * ((W + 31) / 32) < kSubMinWarps) {
      S.subs.clear();
      S.sub_meta.clear();
      S.sub_lrow.clear();
      S.sub_loc.clear();
      S.sub_max_rows = S.sub_max_f = S.sub_max_n = S.sub_max_l = 0;
      S.sub_total = S.sub_members = S.sub_rows_max = 0;
      S.n_levels = F.n_levels;
      level.assign(F.sn_level.begin(), F.sn_level.end());
      inside.assign(F.ns, 0);
    }
    if (WB < 32) {
      build_subtree_packs(F, S, WB, w_lo, w_hi);
      // by default only where the packs fill warps enough (a few hundred subtree packs walk
      // slower than the levels they replace)
      if (!tu.subtree_rows && (int64_t)S.sp_items.size() < kSubPackMinWarps) {
        S = Schedule{};
        S.n_levels = F.n_levels;
        S.ns = F.ns;
        level.assign(F.sn_level.begin(), F.sn_level.end());
        inside.assign(F.ns, 0);
      }
    }
  }
  std::vector<std::vector<int>> by_level(S.n_levels);
  for (int s = 0; s < F.ns; ++s)
    if (!inside[s]) by_level[level[s]].push_back(s);
  auto pack = [](int s, int r0, int r1, int w0, bool partial, int c_lo, int c_hi) {
    return make_int4(s, r0 | (r1 << 16), w0 | ((int)partial << 30), c_lo | (c_hi << 16));
  };
  // Levels with fewer items than can fill the GPU split each dot product into pieces of at
  // least min_piece terms (multiples of the unroll), enough to reach target_warps warps.
  const int nwc = (w_hi - w_lo + WB - 1) / WB;
  auto pieces_of = [&](int len, int split) {
    const int np = std::max(1, std::min(split, len / min_piece));
    const int plen = ((len + np - 1) / np + kUnroll - 1) / kUnroll * kUnroll;
    return std::max(plen, 1);
  };
  S.fwd_ptr.assign(1, 0);
  S.bwd_ptr.assign(1, 0);
  for (int l = 0; l < S.n_levels; ++l) {
    int64_t nfw = 0, nbw = 0;
    for (int s : by_level[l]) {
      const int k = F.sn_k[s], nf = k + F.sn_m[s];
      nfw += (int64_t)((nf + RPI_f - 1) / RPI_f) * nwc;
      nbw += (int64_t)((k + RPI_b - 1) / RPI_b) * nwc;
    }
    const int fsplit = (int)std::max<int64_t>(1, (target_warps + nfw - 1) / std::max<int64_t>(nfw, 1));
    const int bsplit = (int)std::max<int64_t>(1, (target_warps + nbw - 1) / std::max<int64_t>(nbw, 1));
    const bool pack_level = pack_rows > 0 && nfw >= pack_min_warps;
    std::vector<int> packable;
    for (int s : by_level[l]) {
      const int k = F.sn_k[s], nf = k + F.sn_m[s], c0 = F.sn_col0[s];
      if (pack_level && nf <= pack_rows && k <= kPackMaxK && F.sn_rowptr[s] < INT32_MAX) {
        packable.push_back(s);   // the whole supernode in one lane
        continue;
      }
      bool zf_s = false, zb_s = false;
      const int fplen = pieces_of(k, fsplit);
      for (int r0 = 0; r0 < nf; r0 += RPI_f) {
        const int r1 = std::min(nf, r0 + RPI_f), jmax = std::min(k, r1);
        const bool partial = jmax > fplen;
        zf_s |= partial && r0 < k;
        for (int c_lo = 0; c_lo < jmax; c_lo += fplen)
          for (int w0 = w_lo; w0 < w_hi; w0 += WB)
            S.fi.push_back(pack(s, r0, r1, w0, partial, c_lo, std::min(jmax, c_lo + fplen)));
      }
      for (int i0 = 0; i0 < k; i0 += RPI_b) {
        const int i1 = std::min(k, i0 + RPI_b), len = nf - i0;
        const int bplen = pieces_of(len, bsplit);
        const bool partial = len > bplen;
        zb_s |= partial;
        for (int c_lo = i0; c_lo < nf; c_lo += bplen)
          for (int w0 = w_lo; w0 < w_hi; w0 += WB)
            S.bi.push_back(pack(s, i0, i1, w0, partial, c_lo, std::min(nf, c_lo + bplen)));
      }
      if (zf_s) for (int i = 0; i < k; ++i) S.zf.push_back(c0 + i);
      if (zb_s) for (int i = 0; i < k; ++i) S.zb.push_back(c0 + i);
    }
    // similar shapes share a pack (little padding)
    std::stable_sort(packable.begin(), packable.end(), [&](int a, int c) {
      return std::make_pair(F.sn_k[a], F.sn_m[a]) < std::make_pair(F.sn_k[c], F.sn_m[c]);
    });
    // lanes per packed supernode: as tuned, else 4 on levels whose packs would give few warps at
    // one lane each (more warps and shorter chains per lane), 1 on the others
    const int lps = tu.pack_lanes ? tu.pack_lanes
                                  : ((int64_t)(packable.size() + 31) / 32 < kPackLanesWarps ? 4 : 1);
    const int per_pack = 32 / lps;
    for (size_t i = 0; i < packable.size(); i += per_pack) {
      const int count = (int)std::min<size_t>(per_pack, packable.size() - i);
      int NP = 0, KP = 0;
      for (int l = 0; l < count; ++l) {
        const int t = packable[i + l];
        NP = std::max(NP, F.sn_k[t] + F.sn_m[t]);
        KP = std::max(KP, F.sn_k[t]);
      }
      const int NPq = (NP + lps - 1) / lps;
      const int64_t p = (int64_t)S.pack_sn.size() / 32, off = (int64_t)S.pack_vals.size() / 32;
      if (p >= INT32_MAX || off >= INT32_MAX) throw Error(JJA_ERR_ARG, "too many packed supernodes");
      S.pack_vals.resize(S.pack_vals.size() + (size_t)32 * NPq * KP, 0.0);
      double* vals = S.pack_vals.data() + off * 32;
      for (int l = 0; l < 32; ++l) {   // slots: the first `count` of 32 entries
        if (l >= count) {
          S.pack_sn.push_back(-1);
          S.pack_meta.push_back(make_int4(0, 0, 0, 0));
          continue;
        }
        const int t = packable[i + l], k = F.sn_k[t], nf = k + F.sn_m[t];
        S.pack_sn.push_back(t);
        S.pack_meta.push_back(make_int4(F.sn_col0[t], k, nf, (int)F.sn_rowptr[t]));
        const double* Fs = F.fcol.data() + F.sn_valptr[t];
        for (int j = 0; j < k; ++j)
          for (int r = 0; r < nf; ++r) {
            const int lane = l * lps + r % lps, rr = r / lps;
            vals[((int64_t)j * NPq + rr) * 32 + lane] = Fs[(int64_t)j * nf + r];
          }
      }
      const int4 item = make_int4((int)(-1 - p), count, NP | (KP << 16) | (lps << 24), (int)off);
      S.fi.push_back(item);
      S.bi.push_back(item);
    }
    S.level_packed.push_back(!packable.empty());
    S.fwd_ptr.push_back((int64_t)S.fi.size());
    S.bwd_ptr.push_back((int64_t)S.bi.size());
  }
  for (int l = S.n_levels - 1; l >= 0; --l)
    S.bi_flow.insert(S.bi_flow.end(), S.bi.begin() + S.bwd_ptr[l], S.bi.begin() + S.bwd_ptr[l + 1]);
  const int ns = F.ns;
  std::vector<uint32_t> nfi(ns, 0), nbi(ns, 0);
  for (const int4& v : S.fi) for_each_supernode(S, v, [&](int s) { nfi[s]++; });
  for (const int4& v : S.bi) for_each_supernode(S, v, [&](int s) { nbi[s]++; });
  S.fcnt.assign(ns, 0);
  S.bcnt.assign(ns, 0);
  S.fon.assign(ns, -1);
  S.fnot.assign(ns, -1);
  S.bon.assign(ns, -1);
  S.bnot.assign(ns, -1);
  for (int s = 0; s < ns; ++s) {
    const int par = F.sn_parent[s];
    if (par < 0) continue;
    if (par >= ns || F.sn_level[par] <= F.sn_level[s]) throw Error(JJA_ERR_INTERNAL, "supernode levels are not topological");
    S.fcnt[par] += nfi[s];
    S.fnot[s] = par;
    S.bnot[par] = par;
    S.bon[s] = par;
    S.bcnt[s] = nbi[par];
  }
  for (int s = 0; s < ns; ++s)
    if (S.fcnt[s]) S.fon[s] = s;
  return S;
}

// Face <-> junction tables of a cycle matrix (CSR over the original face order, entries +-1), in
// the factor's face order: per permuted face its junction codes (junction << 1) | (entry is -1)
// as CSR (and a fixed-degree copy when every face has at most kEllMax junctions), the original
// face of each permuted face, and per junction its (at most 2) faces (face << 1) | (entry is -1).
struct FaceTables {
  std::vector<int64_t> fj_ptr;
  std::vector<int32_t> fj_col, face_orig, jf_face, ell;
  int deg = 0;
};

FaceTables face_tables(int Nj, int Nf, const int64_t* a_rowptr, const int32_t* a_col, const double* a_val,
                       const std::vector<int>& perm) {
  if (Nj >= (1 << 30) || Nf >= (1 << 30)) throw Error(JJA_ERR_ARG, "too many junctions or faces");
  FaceTables ft;
  ft.fj_ptr.assign(Nf + 1, 0);
  ft.face_orig.resize(Nf);
  ft.jf_face.assign(2 * (size_t)Nj, -1);
  for (int pn = 0; pn < Nf; ++pn) {
    const int f = perm[pn];
    ft.face_orig[pn] = f;
    for (int64_t q = a_rowptr[f]; q < a_rowptr[f + 1]; ++q) {
      const int j = a_col[q];
      const double v = a_val[q];
      if (j < 0 || j >= Nj) throw Error(JJA_ERR_ARG, "cycle matrix column out of range");
      if (v != 1.0 && v != -1.0) throw Error(JJA_ERR_ARG, "cycle matrix entries must be +1 or -1");
      const int neg = v < 0 ? 1 : 0;
      ft.fj_col.push_back((j << 1) | neg);
      const int slot = ft.jf_face[2 * (size_t)j] < 0 ? 0 : (ft.jf_face[2 * (size_t)j + 1] < 0 ? 1 : -1);
      if (slot < 0) throw Error(JJA_ERR_ARG, "a junction lies on more than two faces (non-planar cycle matrix)");
      ft.jf_face[2 * (size_t)j + slot] = (pn << 1) | neg;
    }
    ft.fj_ptr[pn + 1] = (int64_t)ft.fj_col.size();
  }
  for (int pn = 0; pn < Nf; ++pn) ft.deg = std::max<int>(ft.deg, (int)(ft.fj_ptr[pn + 1] - ft.fj_ptr[pn]));
  if (ft.deg >= 1 && ft.deg <= kEllMax) {
    ft.ell.assign((size_t)Nf * ft.deg, -1);
    for (int pn = 0; pn < Nf; ++pn)
      for (int64_t i = ft.fj_ptr[pn]; i < ft.fj_ptr[pn + 1]; ++i)
        ft.ell[(size_t)pn * ft.deg + (i - ft.fj_ptr[pn])] = ft.fj_col[i];
  } else {
    ft.deg = 0;
  }
  return ft;
}

// the face tables into a kernel table set; `up` uploads a host array and returns its device copy
template <class Up>
void set_face_tables(Tables& t, const FaceTables& ft, Up up) {
  t.fj_ptr = up(ft.fj_ptr.data(), ft.fj_ptr.size());
  t.fj_col = up(ft.fj_col.data(), ft.fj_col.size());
  if (ft.deg) {
    t.fj_ell = up(ft.ell.data(), ft.ell.size());
    t.face_deg = ft.deg;
  }
  t.face_orig = up(ft.face_orig.data(), ft.face_orig.size());
  t.jf_face = up(ft.jf_face.data(), ft.jf_face.size());
}


// Every item of a dataflow sweep may only wait for items that come before it in the sweep's
// order, and the counts it waits for must be exactly the number of items that will count.
// Otherwise warps could wait for items no running warp holds.
void check_schedule(const Schedule& S) {
  auto check = [&](const std::vector<int4>& items, const std::vector<int32_t>& on, const std::vector<uint32_t>& cnt,
                   const std::vector<int32_t>& notify, const char* which) {
    const int ns = S.ns;
    std::vector<int64_t> first(ns, INT64_MAX), last_notifier(ns, -1);
    std::vector<uint32_t> notifiers(ns, 0);
    for (int64_t i = 0; i < (int64_t)items.size(); ++i) {
      for_each_supernode(S, items[i], [&](int s) {
        if (s < 0 || s >= ns) throw Error(JJA_ERR_INTERNAL, std::string(which) + ": item supernode out of range");
        first[s] = std::min(first[s], i);
        const int t = notify[s];
        if (t >= 0) {
          last_notifier[t] = i;
          notifiers[t]++;
        }
      });
    }
    for (int s = 0; s < ns; ++s) {
      const int t = on[s];
      if (t < 0) continue;
      if (notifiers[t] != cnt[s])
        throw Error(JJA_ERR_INTERNAL, std::string(which) + ": wait count does not match the items that count");
      if (first[s] != INT64_MAX && last_notifier[t] >= first[s])
        throw Error(JJA_ERR_INTERNAL, std::string(which) + ": an item waits for a later item");
    }
  };
  check(S.fi, S.fon, S.fcnt, S.fnot, "forward schedule");
  check(S.bi_flow, S.bon, S.bcnt, S.bnot, "backward schedule");
}

}  // namespace

namespace {

// {sin, cos}(k pi/32768) in units of 2^-62: first-quadrant values in extended precision,
// rounded once, then exact quadrant symmetries (sin(m pi) and cos(m pi + pi/2) are exactly 0)
std::vector<longlong2> build_sin_table() {
  std::vector<longlong2> tab((size_t)kSinTable);
  const long double pi_l = 3.141592653589793238462643383279502884L;
  const long double scale = 4611686018427387904.0L;   // 2^62
  const int quarter = kSinTable / 4;
  for (int k = 0; k < kSinTable; ++k) {
    const int q = k / quarter, r = k % quarter;
    const long double ang = (long double)r * pi_l / (long double)(kSinTable / 2);
    const long long s0 = llroundl(sinl(ang) * scale), c0 = llroundl(cosl(ang) * scale);
    const long long sv[4] = {s0, c0, -s0, -c0}, cv[4] = {c0, -s0, -c0, s0};
    tab[(size_t)k] = make_longlong2(sv[q], cv[q]);
  }
  return tab;
}

}  // namespace

struct jja_factor {
  std::unique_ptr<jja::Factor> f;
};

// Problems [w0, w0 + wn) stepped as one chain of launches: their work items per level, the rows
// that split dot products accumulate into, their step counters, and their stream (null: the
// caller's). A plan holds the group of all its problems (used by solves, the adjoint and the
// dataflow schedule) and, when it steps its problems in independent groups, those: the groups'
// chains run concurrently, so each fills the SMs the other's level tails and latency-bound
// launches leave idle.
struct Group {
  int w0 = 0, wn = 0;
  std::vector<int64_t> fwd_ptr, bwd_ptr;
  std::vector<char> level_packed;
  int4* fwd_items = nullptr;
  int4* bwd_items = nullptr;        // levels ascending (level launches index them per level)
  int32_t* zrows_f = nullptr;       // rows of z accumulated by partial forward items
  int32_t* zrows_b = nullptr;       // rows of x accumulated by partial backward items
  int nz_f = 0, nz_b = 0;
  int64_t* d_step = nullptr;        // step counters (see StepArgs)
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;       // end of the group's chain in a call (joined by the caller's stream)
};

struct jja_plan {
  int Nj = 0, Nf = 0, W = 0, width = 3, WB = 1, n_levels = 0;
  int rows_per_lane = kDefaultRowsPerLane, rows_per_lane_fwd = kDefaultRowsPerLane;   // backward, forward
  bool pdl = false;   // step kernels launched with programmatic dependent launch
  double dt = 0.0, extrap[4] = {0, 0, 0, 0};
  Tables t{};
  FactorDev F{};
  std::vector<void*> allocs;
  Group all;                        // all W problems
  std::vector<Group> groups;        // the step's independent groups (empty: one, `all`)
  cudaEvent_t fork = nullptr;       // start of a call on the caller's stream (the groups wait on it)
  int4* bwd_flow_items = nullptr;   // the backward items of `all` root first (dataflow sweep order)
  double *b = nullptr, *z = nullptr, *x = nullptr, *xj = nullptr;
  int32_t* perm = nullptr;   // new -> old face
  double* isq = nullptr;        // Is / c0 (Nj x W)
  int resistive = 0;
  // dataflow sweeps (schedule 2): dependency tables per supernode, counters, error flag
  int flow = 0, ns = 0;
  const int32_t* f_wait_on = nullptr;
  const uint32_t* f_wait_count = nullptr;
  const int32_t* f_notify = nullptr;
  const int32_t* b_wait_on = nullptr;
  const uint32_t* b_wait_count = nullptr;
  const int32_t* b_notify = nullptr;
  unsigned* counters = nullptr;   // forward: [next, done[ns]], then backward: [next, done[ns]]
  int* flow_err = nullptr;
  int flow_blocks[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};   // resident blocks per (rows/lane 2,4,8,1) x (bwd, fwd)
  // cooperative sweeps (schedule 3): level boundaries of `all` on the device, blocks per launch
  // ([backward, forward][without, with W = 1 packs]), barrier arrival counters [backward, forward]
  int coop = 0;
  int64_t* coop_fwd_lp = nullptr;
  int64_t* coop_bwd_lp = nullptr;
  int coop_grid[2][2] = {{0, 0}, {0, 0}};
  unsigned* coop_bar = nullptr;
  bool coop_packs = false;
  // fast Poisson solve of uniform square arrays (jja_plan_set_fast_poisson): replaces both sweeps
  SubDev sub{};        // subtree sweeps (k_subtree; n = 0: none)
  SubPackDev subp{};   // W = 1 subtree packs (k_subtree_pack; n_items = 0: none)
  int dst = 0;
  int dst_lines = 0;   // grid lines per block of the sine-transform kernels (0: by grid size)
  DstArgs dst_args{};
  std::vector<int32_t> iperm_host;   // original face -> factor's face order
  int64_t bytes = 0;
  // captured graphs of a fixed-length step sequence, keyed by the buffers they bake in (a few
  // are kept: double-buffered source windows alternate between two keys), most recent last
  struct CachedGraph {
    std::vector<uint64_t> key;
    cudaGraphExec_t exec;
  };
  std::vector<CachedGraph> graphs;
  std::vector<CachedGraph> adj_graphs;   // adjoint segment walks
  static constexpr size_t kMaxGraphs = 16;   // 5 graph lengths x two alternating source windows fit
  ~jja_plan() {
    for (auto& g : graphs) cudaGraphExecDestroy(g.exec);
    for (auto& g : adj_graphs) cudaGraphExecDestroy(g.exec);
    for (Group& g : groups) {
      if (g.stream) cudaStreamDestroy(g.stream);
      if (g.done) cudaEventDestroy(g.done);
    }
    if (fork) cudaEventDestroy(fork);
    for (void* p : allocs) cudaFree(p);
  }
  template <class T>
  T* up(const T* h, size_t n) {
    T* d = upload(h, n, bytes);
    allocs.push_back(d);
    return d;
  }
};

namespace {

// Launch with programmatic stream serialisation (the kernel overlaps its launch with the tail
// of the previous kernel of the stream; it synchronises itself in pdl_begin), or plainly.
template <typename... KArgs, typename... Args>
void launch(bool pdl, void (*kernel)(KArgs...), int grid, int block, cudaStream_t st, Args... args) {
  if (!pdl) {
    kernel<<<grid, block, 0, st>>>(args...);
  } else {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    JJA_CUDA(cudaLaunchKernelEx(&cfg, kernel, args...));
  }
  g_launches++;
}

// the same with a 2-D grid and dynamic shared memory
template <typename... KArgs, typename... Args>
void launch_smem(bool pdl, void (*kernel)(KArgs...), dim3 grid, int block, size_t smem, cudaStream_t st,
                 Args... args) {
  if (!pdl) {
    kernel<<<grid, block, smem, st>>>(args...);
  } else {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    JJA_CUDA(cudaLaunchKernelEx(&cfg, kernel, args...));
  }
  g_launches++;
}

// the cooperative sweep kernel of a rows-per-lane variant (for occupancy queries)
const void* coop_kernel(int rpl, bool forward, bool packs) {
#define JJA_COOP_K(R) \
  (forward ? (packs ? (const void*)k_coop_sweep<R, true, true> : (const void*)k_coop_sweep<R, true, false>) \
           : (packs ? (const void*)k_coop_sweep<R, false, true> : (const void*)k_coop_sweep<R, false, false>))
  switch (rpl) {
    case 1: return JJA_COOP_K(1);
    case 2: return JJA_COOP_K(2);
    case 8: return JJA_COOP_K(8);
    default: return JJA_COOP_K(4);
  }
#undef JJA_COOP_K
}

// zero the rows that partial items of the coming sweep accumulate into (and, for a dataflow
// sweep, its counters)
void launch_zero_rows(jja_plan* p, const Group& g, cudaStream_t st, bool forward, double* v) {
  if (p->coop) return;   // a cooperative sweep zeroes its rows in its first phase
  const int n = forward ? g.nz_f : g.nz_b;
  const int n_ctr = p->flow ? p->ns + 1 : 0;
  if (!n && !n_ctr) return;
  unsigned* ctr = p->flow ? p->counters + (forward ? 0 : p->ns + 1) : nullptr;
  launch(p->pdl, k_zero_rows, grid_for(std::max<int64_t>((int64_t)n * g.wn, n_ctr), 256), 256, st, v,
         (const int32_t*)(forward ? g.zrows_f : g.zrows_b), n, p->W, g.w0, g.wn, ctr, n_ctr);
}

void launch_zero_rows(jja_plan* p, cudaStream_t st, bool forward, double* v) { launch_zero_rows(p, p->all, st, forward, v); }

// the dataflow sweep: all problems in one persistent launch (the schedule of `all`)
template <int RPL>
void launch_flow(jja_plan* p, cudaStream_t st, bool forward, double* b, double* z, double* x,
                 const uint32_t* wait_count_override = nullptr) {
  const int vi = RPL == 2 ? 0 : (RPL == 4 ? 1 : (RPL == 8 ? 2 : 3));   // index into flow_blocks
  Flow fl;
  unsigned* base = p->counters + (forward ? 0 : p->ns + 1);
  fl.next = reinterpret_cast<int*>(base);
  fl.done = base + 1;
  fl.wait_on = forward ? p->f_wait_on : p->b_wait_on;
  fl.wait_count = wait_count_override ? wait_count_override : (forward ? p->f_wait_count : p->b_wait_count);
  fl.notify = forward ? p->f_notify : p->b_notify;
  fl.err = p->flow_err;
  const int n = (int)(forward ? p->all.fwd_ptr.back() : p->all.bwd_ptr.back());
  if (!n) return;
  const int grid = std::max(1, std::min((n + kWarpsPerBlock - 1) / kWarpsPerBlock, p->flow_blocks[vi][forward]));
  if (forward)
    launch(p->pdl, k_flow_sweep<RPL, true>, grid, kWarpsPerBlock * 32, st, p->F, (const int4*)p->all.fwd_items, n,
           p->W, p->WB, b, z, x, fl);
  else
    launch(p->pdl, k_flow_sweep<RPL, false>, grid, kWarpsPerBlock * 32, st, p->F, (const int4*)p->bwd_flow_items, n,
           p->W, p->WB, b, z, x, fl);
}

// a sweep as one cooperative launch over all levels (schedule 3; the group of all problems)
template <int RPL>
void launch_coop(jja_plan* p, cudaStream_t st, bool forward, double* b, double* z, double* x,
                 unsigned unreachable = 0) {
  const Group& g = p->all;
  const bool packs = p->coop_packs;
  void (*kern)(FactorDev, const int4*, const int64_t*, int, int, int, double*, double*, double*, const int32_t*, int,
               int, int, unsigned*, unsigned*, int*, unsigned);
  if (forward) kern = packs ? k_coop_sweep<RPL, true, true> : k_coop_sweep<RPL, true, false>;
  else kern = packs ? k_coop_sweep<RPL, false, true> : k_coop_sweep<RPL, false, false>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)p->coop_grid[forward][packs]);
  cfg.blockDim = dim3((unsigned)kCoopThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  JJA_CUDA(cudaLaunchKernelEx(&cfg, kern, p->F, (const int4*)(forward ? g.fwd_items : g.bwd_items),
                              (const int64_t*)(forward ? p->coop_fwd_lp : p->coop_bwd_lp), p->n_levels, p->W, p->WB, b,
                              z, x, (const int32_t*)(forward ? g.zrows_f : g.zrows_b), forward ? g.nz_f : g.nz_b, g.w0,
                              g.wn, p->coop_bar + (forward ? 1 : 0), p->coop_bar + (forward ? 0 : 1), p->flow_err,
                              unreachable));
  g_launches++;
}

// the subtree sweep of group g (before the forward levels, after the backward ones)
void launch_subtrees(jja_plan* p, const Group& g, cudaStream_t st, bool forward, double* b, double* z, double* x) {
  if (p->subp.n_items) {
    const int grid = (p->subp.n_items + kSubPackWarps - 1) / kSubPackWarps;
    const size_t smem = (size_t)kSubPackWarps * p->subp.max_rows * 32 * sizeof(double);
    launch_smem(p->pdl, sub_pack_kernel(forward, p->subp.ns), dim3((unsigned)grid), kSubPackWarps * 32, smem, st,
                p->F, p->subp, p->W, b, z, x);
  }
  if (!p->sub.n) return;
  const int blocks = (g.wn + 31) / 32;
  const int warps = std::min(blocks, kSubMaxWarps);
  const dim3 grid((unsigned)p->sub.n, (unsigned)((blocks + warps - 1) / warps));
  const size_t smem = sub_smem_bytes(p->sub, warps);
  launch_smem(p->pdl, forward ? k_subtree<true> : k_subtree<false>, grid, warps * 32, smem, st, p->F, p->sub, p->W,
              g.w0, g.wn, b, z, x);
}

template <int RPL>
void launch_sweep(jja_plan* p, const Group& g, cudaStream_t st, bool forward, double* b, double* z, double* x) {
  if (p->flow) {
    launch_flow<RPL>(p, st, forward, b, z, x);
    return;
  }
  if (p->coop) {
    launch_coop<RPL>(p, st, forward, b, z, x);
    return;
  }
  if (forward) {  // levels ascending (children before parents); b is consumed, z produced
    launch_subtrees(p, g, st, true, b, z, x);
    for (int l = 0; l < p->n_levels; ++l) {
      const int n = (int)(g.fwd_ptr[l + 1] - g.fwd_ptr[l]);
      if (!n) continue;
      launch(p->pdl, g.level_packed[l] ? k_fwd_level<RPL, true> : k_fwd_level<RPL, false>,
             (n + kWarpsPerBlock - 1) / kWarpsPerBlock, kWarpsPerBlock * 32, st, p->F,
             (const int4*)(g.fwd_items + g.fwd_ptr[l]), n, p->W, p->WB, b, z);
    }
  } else {        // levels descending; x produced
    for (int l = p->n_levels - 1; l >= 0; --l) {
      const int n = (int)(g.bwd_ptr[l + 1] - g.bwd_ptr[l]);
      if (!n) continue;
      launch(p->pdl, g.level_packed[l] ? k_bwd_level<RPL, true> : k_bwd_level<RPL, false>,
             (n + kWarpsPerBlock - 1) / kWarpsPerBlock, kWarpsPerBlock * 32, st, p->F,
             (const int4*)(g.bwd_items + g.bwd_ptr[l]), n, p->W, p->WB, (const double*)z, x);
    }
    launch_subtrees(p, g, st, false, b, z, x);
  }
}

// one triangular sweep over the levels with the plan's rows-per-lane variant of the kernels
void launch_sweep_any(jja_plan* p, const Group& g, cudaStream_t st, bool forward, double* b, double* z, double* x) {
  switch (forward ? p->rows_per_lane_fwd : p->rows_per_lane) {
    case 1: launch_sweep<1>(p, g, st, forward, b, z, x); break;
    case 2: launch_sweep<2>(p, g, st, forward, b, z, x); break;
    case 8: launch_sweep<8>(p, g, st, forward, b, z, x); break;
    default: launch_sweep<4>(p, g, st, forward, b, z, x); break;
  }
}

void launch_sweep_any(jja_plan* p, cudaStream_t st, bool forward, double* b, double* z, double* x) {
  launch_sweep_any(p, p->all, st, forward, b, z, x);
}

void launch_levels(jja_plan* p, const Group& g, cudaStream_t st, bool forward) {
  launch_zero_rows(p, g, st, forward, forward ? p->z : p->x);
  launch_sweep_any(p, g, st, forward, p->b, p->z, p->x);
}


// x = K^-1 b for group g: the two triangular sweeps, or the three sine-transform kernels
void launch_face_solve(jja_plan* p, const Group& g, cudaStream_t st) {
  if (!p->dst) {
    launch_levels(p, g, st, true);
    launch_levels(p, g, st, false);
    return;
  }
  const DstArgs& d = p->dst_args;
  // an FFT buffer of 2 (m + 1) complex points, two lines of m values, m + 1 twiddles
  const size_t smx = (size_t)3 * (d.mx + 1) * sizeof(double2) + (size_t)2 * d.mx * sizeof(double);
  const size_t smy = (size_t)3 * (d.my + 1) * sizeof(double2) + (size_t)2 * d.my * sizeof(double);
  const int tx = std::min(512, d.mx + 1), ty = std::min(512, d.my + 1);
  // two lines per block halve the butterflies but also the blocks: pair only while the
  // smaller grid still fills every SM twice
  const int lines = p->dst_lines ? p->dst_lines
                                 : ((int64_t)((std::min(d.mx, d.my) + 1) / 2) * g.wn >= 2 * kNumSMs ? 2 : 1);
  const unsigned row_blocks = (unsigned)((d.my + lines - 1) / lines), col_blocks = (unsigned)((d.mx + lines - 1) / lines);
  k_dst_rows<<<dim3(row_blocks, (unsigned)g.wn), tx, smx, st>>>(d, p->b, d.t1, p->W, g.w0, 1, 0, lines);
  k_dst_cols<<<dim3(col_blocks, (unsigned)g.wn), ty, smy, st>>>(d, g.w0, lines);
  k_dst_rows<<<dim3(row_blocks, (unsigned)g.wn), tx, smx, st>>>(d, d.t2, p->x, p->W, g.w0, 0, 1, lines);
  g_launches += 3;
}

void launch_face_solve(jja_plan* p, cudaStream_t st) { launch_face_solve(p, p->all, st); }

// q of the first step of a run, from the phase history (the args' group of problems)
void launch_junction(jja_plan* p, StepArgs& a, cudaStream_t st) {
  launch(p->pdl, k_junction, grid_for((int64_t)p->Nj * a.wn, 256), 256, st, a, p->t, p->xj);
}

// one time step of group g whose q is already in p->xj; `fuse_next` also leaves the next step's
// q there. With `ev` (5 events) the boundaries face rhs | forward | backward | update(+next q)
// are recorded.
void launch_step(jja_plan* p, const Group& g, StepArgs& a, cudaStream_t st, bool fuse_next,
                 cudaEvent_t* ev = nullptr) {
  const int64_t nj = (int64_t)p->Nj * g.wn, nf = (int64_t)p->Nf * g.wn;
  if (ev) JJA_CUDA(cudaEventRecord(ev[0], st));
  launch(p->pdl, k_face_rhs, grid_for(nf, 256), 256, st, a, p->t, (const double*)p->xj, p->b);
  if (ev) JJA_CUDA(cudaEventRecord(ev[1], st));
  if (p->dst) {
    launch_face_solve(p, g, st);
    if (ev) JJA_CUDA(cudaEventRecord(ev[2], st));
  } else {
    launch_levels(p, g, st, true);
    if (ev) JJA_CUDA(cudaEventRecord(ev[2], st));
    launch_levels(p, g, st, false);
  }
  if (ev) JJA_CUDA(cudaEventRecord(ev[3], st));
  if (fuse_next) launch(p->pdl, k_update<true>, grid_for(nj, 256), 256, st, a, p->t, p->xj, (const double*)p->x);
  else launch(p->pdl, k_update<false>, grid_for(nj, 256), 256, st, a, p->t, p->xj, (const double*)p->x);
  if (ev) JJA_CUDA(cudaEventRecord(ev[4], st));
}

StepArgs make_args(jja_plan* p, jja_state* s, const Group& g) {
  StepArgs a{};
  a.Nj = p->Nj; a.Nf = p->Nf; a.W = p->W; a.width = p->width;
  a.w0 = g.w0; a.wn = g.wn;
  for (int k = 0; k < 4; ++k) { a.h[k] = s->hist[k]; a.e[k] = p->extrap[k]; }
  a.theta_s = s->theta_s;
  a.Is = s->Is; a.f = s->f; a.Vs = s->Vs; a.T = s->T;
  a.noise_mode = s->noise_mode;
  a.noise = s->noise;
  a.seed = s->seed;
  a.d_step = g.d_step;
  a.th_out = s->th_out;
  a.I_out = s->I_out;
  a.store_all = s->store_all ? 1 : 0;
  a.dt = p->dt;
  a.Isq = (s->Is.ptr && !s->Is.stride_t) ? jja_view{p->isq, p->W, 1, 0} : jja_view{nullptr, 0, 0, 0};
  a.resistive = p->resistive;
  return a;
}

// refresh Is / c0 from a time-independent current-source view (before the first step of a run)
void launch_scale_sources(jja_plan* p, jja_state* s, cudaStream_t st) {
  if (!s->Is.ptr || s->Is.stride_t) return;
  launch(p->pdl, k_scale_sources, grid_for((int64_t)p->Nj * p->W, 256), 256, st, s->Is, p->t.inv_c0, p->isq, p->Nj,
         p->W);
}

// rotate the history: the oldest buffer receives theta_next
void rotate(jja_state* s, int width) {
  const int nh = width - 1;
  double* oldest = s->hist[nh - 1];
  for (int k = nh - 1; k > 0; --k) s->hist[k] = s->hist[k - 1];
  s->hist[0] = oldest;
}

// time-dependent sources must cover steps [step, step + nsteps)
void check_window(const jja_state* s, int nsteps, const char* who) {
  const jja_view* v[4] = {&s->Is, &s->f, &s->Vs, &s->T};
  for (const jja_view* x : v) {
    if (!x->ptr || !x->stride_t) continue;
    if (s->step < s->src_t0 || s->step + nsteps > s->src_t0 + s->src_steps)
      throw Error(JJA_ERR_ARG, std::string(who) + ": steps [" + std::to_string(s->step) + ", " +
                                   std::to_string(s->step + nsteps) + ") are outside the source window [" +
                                   std::to_string(s->src_t0) + ", " + std::to_string(s->src_t0 + s->src_steps) + ")");
  }
}

// the groups a call steps: the plan's independent groups, or the group of all problems
std::vector<Group*> step_groups(jja_plan* p) {
  std::vector<Group*> gs;
  if (p->groups.empty()) gs.push_back(&p->all);
  for (Group& g : p->groups) gs.push_back(&g);
  return gs;
}

// the stream group g runs on in a call on the caller's stream st
cudaStream_t stream_of(const Group& g, cudaStream_t st) { return g.stream ? g.stream : st; }

// fork: the groups' own streams wait for the caller's stream; join: the caller's stream waits
// for them. Every call joins before it returns, so work the caller queues next is ordered after
// all groups.
void fork_groups(jja_plan* p, cudaStream_t st) {
  if (p->groups.size() < 2) return;
  JJA_CUDA(cudaEventRecord(p->fork, st));
  for (Group& g : p->groups)
    if (g.stream) JJA_CUDA(cudaStreamWaitEvent(g.stream, p->fork, 0));
}

void join_groups(jja_plan* p, cudaStream_t st) {
  if (p->groups.size() < 2) return;
  for (Group& g : p->groups) {
    if (!g.stream) continue;
    JJA_CUDA(cudaEventRecord(g.done, g.stream));
    JJA_CUDA(cudaStreamWaitEvent(st, g.done, 0));
  }
}

void set_counters(jja_plan* p, const jja_state* s, cudaStream_t st) {
  for (Group* g : step_groups(p)) launch(p->pdl, k_set_counters, 1, 1, st, g->d_step, s->step, s->src_t0);
}

// graph of G fused steps for the state's current buffers (captured on first use, then cached);
// with several groups the graph forks into their streams and joins back
cudaGraphExec_t graph_for(jja_plan* p, const jja_state* s, cudaStream_t st, int G) {
  std::vector<uint64_t> key = {(uint64_t)s->hist[0], (uint64_t)s->hist[1], (uint64_t)s->hist[2],
                               (uint64_t)s->hist[3], (uint64_t)s->theta_s, (uint64_t)s->noise_mode, s->seed,
                               (uint64_t)st, (uint64_t)G, (uint64_t)s->store_all,
                               (uint64_t)(s->store_all ? s->th_out : nullptr),
                               (uint64_t)(s->store_all ? s->I_out : nullptr)};
  for (const jja_view* v : {&s->Is, &s->f, &s->Vs, &s->T}) {
    key.push_back((uint64_t)v->ptr);
    key.push_back((uint64_t)v->stride_n);
    key.push_back((uint64_t)v->stride_w);
    key.push_back((uint64_t)v->stride_t);
  }
  for (size_t k = 0; k < p->graphs.size(); ++k) {
    if (p->graphs[k].key != key) continue;
    jja_plan::CachedGraph hit = p->graphs[k];
    p->graphs.erase(p->graphs.begin() + k);
    p->graphs.push_back(hit);
    return hit.exec;
  }
  if (p->graphs.size() >= jja_plan::kMaxGraphs) {
    cudaGraphExecDestroy(p->graphs.front().exec);
    p->graphs.erase(p->graphs.begin());
  }
  const int period = p->width - 1;
  cudaGraph_t g;
  const std::vector<Group*> gs = step_groups(p);
  JJA_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  fork_groups(p, st);
  for (Group* grp : gs) {   // each group's chain of G steps (the history rotation is the same for all)
    jja_state tmp = *s;
    for (int q = 0; q < G; ++q) {
      StepArgs a = make_args(p, &tmp, *grp);
      a.hout = tmp.hist[period - 1];
      a.th_slot = a.I_slot = -1;
      launch_step(p, *grp, a, stream_of(*grp, st), true);
      rotate(&tmp, p->width);
    }
  }
  join_groups(p, st);
  JJA_CUDA(cudaStreamEndCapture(st, &g));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) throw Error(JJA_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
  p->graphs.push_back({key, exec});
  return exec;
}

}  // namespace

extern "C" {

const char* jja_last_error(void) { return g_err.c_str(); }
int64_t jja_launch_count(void) { return g_launches.load(); }

int jja_factor_create(int n, const int64_t* colptr, const int32_t* rowind, const double* val, const double* cx,
                      const double* cy, const int32_t* perm, const jja_factor_opts* opts, jja_factor** out) {
  return guarded([&] {
    if (!out || !colptr || !rowind || !val || n <= 0) throw Error(JJA_ERR_ARG, "jja_factor_create: bad arguments");
    jja::FactorOptions o;
    if (opts) {
      if (opts->nd_leaf > 0) o.nd_leaf = opts->nd_leaf;
      o.max_supernode = opts->max_supernode;
      o.keep_factor = opts->keep_factor;
      if (opts->relax_zeros >= 0) o.relax_zeros = opts->relax_zeros;
      if (opts->relax_frac >= 0.0) o.relax_frac = opts->relax_frac;
    }
    std::unique_ptr<jja_factor> f(new jja_factor);
    try {
      f->f.reset(jja::factor_create(n, colptr, rowind, val, cx, cy, perm, o));
    } catch (const std::runtime_error& e) {
      const std::string msg = e.what();
      throw Error(msg.find("positive definite") != std::string::npos ? JJA_ERR_NOT_SPD : JJA_ERR_ARG, msg);
    }
    *out = f.release();
  });
}

void jja_factor_destroy(jja_factor* f) { delete f; }

int jja_factor_get_stats(const jja_factor* f, jja_factor_stats* out) {
  return guarded([&] {
    if (!f || !out) throw Error(JJA_ERR_ARG, "null argument");
    const jja::Factor& F = *f->f;
    out->n = F.n;
    out->n_supernodes = F.ns;
    out->n_levels = F.n_levels;
    out->max_k = F.ns ? *std::max_element(F.sn_k.begin(), F.sn_k.end()) : 0;
    out->max_m = F.ns ? *std::max_element(F.sn_m.begin(), F.sn_m.end()) : 0;
    out->nnz_L = F.nnz_L;
    out->f_values = (int64_t)F.fcol.size();
    out->factor_flops = F.factor_flops;
  });
}

int jja_factor_get_perm(const jja_factor* f, int32_t* perm_out) {
  return guarded([&] {
    if (!f || !perm_out) throw Error(JJA_ERR_ARG, "null argument");
    std::copy(f->f->perm.begin(), f->f->perm.end(), perm_out);
  });
}

int jja_factor_get_supernodes(const jja_factor* f, int32_t* col0, int32_t* k, int32_t* m, int32_t* level,
                              int32_t* parent) {
  return guarded([&] {
    if (!f) throw Error(JJA_ERR_ARG, "null factor");
    const jja::Factor& F = *f->f;
    if (col0) std::copy(F.sn_col0.begin(), F.sn_col0.end(), col0);
    if (k) std::copy(F.sn_k.begin(), F.sn_k.end(), k);
    if (m) std::copy(F.sn_m.begin(), F.sn_m.end(), m);
    if (level) std::copy(F.sn_level.begin(), F.sn_level.end(), level);
    if (parent) std::copy(F.sn_parent.begin(), F.sn_parent.end(), parent);
  });
}

int jja_factor_solve_host(const jja_factor* f, double* b, int nrhs) {
  return guarded([&] {
    if (!f || !b || nrhs <= 0) throw Error(JJA_ERR_ARG, "bad arguments");
    jja::factor_solve_host(*f->f, b, nrhs);
  });
}

int jja_factor_check_schedule(const jja_factor* f, int W, const jja_solve_tuning* tuning, int64_t* n_fwd_items,
                              int64_t* n_bwd_items) {
  return guarded([&] {
    if (!f) throw Error(JJA_ERR_ARG, "jja_factor_check_schedule: null factor");
    jja_solve_tuning tu{};
    if (tuning) tu = *tuning;
    const Schedule S = build_schedule(*f->f, W, tu);
    check_schedule(S);
    if (n_fwd_items) *n_fwd_items = (int64_t)S.fi.size();
    if (n_bwd_items) *n_bwd_items = (int64_t)S.bi_flow.size();
  });
}

int jja_factor_schedule_stats(const jja_factor* f, int W, const jja_solve_tuning* tuning, jja_schedule_stats* out) {
  return guarded([&] {
    if (!f || !out) throw Error(JJA_ERR_ARG, "jja_factor_schedule_stats: null argument");
    jja_solve_tuning tu{};
    if (tuning) tu = *tuning;
    const Schedule S = build_schedule(*f->f, W, tu);
    jja_schedule_stats st{};
    st.n_levels = S.n_levels;
    st.n_subtrees = S.sub_total;
    st.n_subtree_members = S.sub_members;
    st.max_subtree_rows = S.sub_rows_max;
    st.n_pack_items = (int)S.sp_items.size();
    st.n_pack_shapes = (int)S.sp_shapes.size();
    st.n_fwd_items = (int64_t)S.fi.size();
    st.n_bwd_items = (int64_t)S.bi.size();
    *out = st;
  });
}

int jja_plan_create(const jja_plan_desc* d, const jja_factor* fac, jja_plan** out) {
  return guarded([&] {
    if (!d || !fac || !out) throw Error(JJA_ERR_ARG, "jja_plan_create: null argument");
    const jja::Factor& F = *fac->f;
    if (d->Nf != F.n) throw Error(JJA_ERR_ARG, "jja_plan_create: factor order != Nf");
    if (d->W <= 0 || d->Nj <= 0) throw Error(JJA_ERR_ARG, "jja_plan_create: W and Nj must be positive");
    if (d->stencil_width < 3 || d->stencil_width > 5) throw Error(JJA_ERR_ARG, "stencil width must be 3, 4 or 5");
    std::unique_ptr<jja_plan> p(new jja_plan);
    p->Nj = d->Nj; p->Nf = d->Nf; p->W = d->W; p->width = d->stencil_width; p->dt = d->dt;
    for (int k = 0; k < 4; ++k) p->extrap[k] = d->extrap[k];
    // launch shape of the triangular solves (jja_solve_tuning; 0 = default), validated again
    // by build_schedule
    const jja_solve_tuning& tu = d->tuning;
    p->WB = resolve_rhs_block(d->W, tu);
    p->rows_per_lane = rows_per_lane_of(tu, false, d->W, F.n);
    p->rows_per_lane_fwd = rows_per_lane_of(tu, true, d->W, F.n);
    p->pdl = tu.pdl == 1;
    p->dst_lines = tu.dst_lines;
    const int Nj = d->Nj, Nf = d->Nf;
    const FaceTables ft = face_tables(Nj, Nf, d->a_rowptr, d->a_col, d->a_val, F.perm);
    {
      // coefficients multiplied by 1/c0 once on the host (the junction kernels then need no
      // final multiply). "resistive": width 3 and c2 = Cv = 0 everywhere, in which case
      // c1 = -Rv - 2 Cv = -c0 exactly and c1/c0 = -1 (time_evolution.py:477-478, 489)
      const int nk = d->stencil_width - 1;
      const size_t nic = d->Ic_w ? (size_t)Nj * d->W : (size_t)Nj;
      std::vector<double> icq(nic), ic(nic), coefq((size_t)nk * Nj), rvq(Nj);
      bool resistive = d->stencil_width == 3;
      for (int j = 0; j < Nj; ++j) {
        const double ic0 = d->inv_c0[j];
        if (d->Ic_w) {
          for (int w = 0; w < d->W; ++w) {
            ic[(size_t)j * d->W + w] = d->Ic_w[(size_t)j * d->W + w];
            icq[(size_t)j * d->W + w] = d->Ic_w[(size_t)j * d->W + w] * ic0;
          }
        } else {
          ic[j] = d->Ic[j];
          icq[j] = d->Ic[j] * ic0;
        }
        rvq[j] = d->Rv[j] * ic0 * ic0;
        for (int k = 0; k < nk; ++k) coefq[(size_t)k * Nj + j] = d->coef[(size_t)k * Nj + j] * ic0;
        if (resistive) resistive = d->coef[(size_t)Nj + j] == 0.0;
      }
      p->resistive = resistive ? 1 : 0;
      p->t.ic_per_w = d->Ic_w ? 1 : 0;
      p->t.Ic = p->up(ic.data(), ic.size());
      p->t.Icq = p->up(icq.data(), icq.size());
      p->t.coefq = p->up(coefq.data(), coefq.size());
      p->t.coef = p->up(d->coef, (size_t)nk * Nj);
      p->t.Rvq = p->up(rvq.data(), rvq.size());
    }
    p->t.inv_c0 = p->up(d->inv_c0, Nj);
    set_face_tables(p->t, ft, [&](auto* h, size_t n) { return p->up(h, n); });
    p->perm = p->up(F.perm.data(), F.perm.size());
    p->iperm_host.assign(F.iperm.begin(), F.iperm.end());
    {
      const std::vector<longlong2> tab = build_sin_table();
      p->t.sincos = p->up(tab.data(), tab.size());
    }
    // factor blocks (column-major copy for the forward pass, row-major for the backward pass)
    std::vector<double> frow(F.fcol.size());
    for (int s = 0; s < F.ns; ++s) {
      const int k = F.sn_k[s], nf = k + F.sn_m[s];
      const double* src = F.fcol.data() + F.sn_valptr[s];
      double* dst = frow.data() + F.sn_valptr[s];
      for (int j = 0; j < k; ++j)
        for (int r = 0; r < nf; ++r) dst[(int64_t)r * k + j] = src[(int64_t)j * nf + r];
    }
    p->F.col0 = p->up(F.sn_col0.data(), F.ns);
    p->F.k = p->up(F.sn_k.data(), F.ns);
    p->F.m = p->up(F.sn_m.data(), F.ns);
    p->F.rowptr = p->up(F.sn_rowptr.data(), F.sn_rowptr.size());
    p->F.rows = p->up(F.rows.data(), F.rows.size());
    p->F.valptr = p->up(F.sn_valptr.data(), F.sn_valptr.size());
    p->F.fcol = p->up(F.fcol.data(), F.fcol.size());
    p->F.frow = p->up(frow.data(), frow.size());
    // work items and dataflow dependencies (built and checked on the host)
    const Schedule S = build_schedule(F, d->W, tu);
    check_schedule(S);
    p->n_levels = S.n_levels;
    auto set_group = [&](Group& g, const Schedule& Sg, int w0, int wn) {
      g.w0 = w0;
      g.wn = wn;
      g.fwd_ptr = Sg.fwd_ptr;
      g.bwd_ptr = Sg.bwd_ptr;
      g.level_packed = Sg.level_packed;
      g.fwd_items = p->up(Sg.fi.data(), Sg.fi.size());
      g.bwd_items = p->up(Sg.bi.data(), Sg.bi.size());
      g.nz_f = (int)Sg.zf.size();
      g.nz_b = (int)Sg.zb.size();
      g.zrows_f = p->up(Sg.zf.data(), Sg.zf.size());
      g.zrows_b = p->up(Sg.zb.data(), Sg.zb.size());
      g.d_step = p->up<int64_t>(nullptr, 4);
      JJA_CUDA(cudaMemset(g.d_step, 0, 4 * sizeof(int64_t)));
    };
    set_group(p->all, S, 0, d->W);
    if (!S.sp_items.empty()) {
      SubPackDev& sp = p->subp;
      sp.items = p->up(S.sp_items.data(), S.sp_items.size());
      sp.shapes = p->up(S.sp_shapes.data(), S.sp_shapes.size());
      sp.meta = p->up(S.sp_meta.data(), S.sp_meta.size());
      sp.lrow = p->up(S.sp_lrow.data(), S.sp_lrow.size());
      sp.loc = p->up(S.sp_loc.data(), S.sp_loc.size());
      sp.c0 = p->up(S.sp_c0.data(), S.sp_c0.size());
      sp.roff = p->up(S.sp_roff.data(), S.sp_roff.size());
      sp.vals = p->up(S.sp_vals.data(), S.sp_vals.size());
      sp.n_items = (int)S.sp_items.size();
      sp.max_rows = S.sp_max_rows;
      sp.ns = S.sp_ns;
      // the attribute is the kernel's, shared by every plan: the largest any plan can need
      const int smem = (int)((size_t)kSubPackWarps * kSubMaxRows * 32 * sizeof(double));
      for (int fw = 0; fw < 2; ++fw)
        JJA_CUDA(cudaFuncSetAttribute(sub_pack_kernel(fw != 0, sp.ns), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      smem));
    }
    if (!S.subs.empty()) {
      SubDev& sd = p->sub;
      sd.tab = p->up(S.subs.data(), S.subs.size());
      sd.meta = p->up(S.sub_meta.data(), S.sub_meta.size());
      sd.lrow = p->up(S.sub_lrow.data(), S.sub_lrow.size());
      sd.loc = p->up(S.sub_loc.data(), S.sub_loc.size());
      sd.n = (int)S.subs.size();
      sd.max_rows = S.sub_max_rows;
      sd.max_f = S.sub_max_f;
      sd.max_n = S.sub_max_n;
      sd.max_l = S.sub_max_l;
      // the attribute is the kernel's, shared by every plan: the largest any plan can need
      SubDev bound{};
      bound.max_rows = kSubMaxRows;
      bound.max_f = kSubMaxF;
      bound.max_n = kSubMaxRows;
      bound.max_l = kSubMaxL;
      const size_t smem = sub_smem_bytes(bound, kSubMaxWarps);
      if (sub_smem_bytes(sd, kSubMaxWarps) > smem || smem > (size_t)227 * 1024)
        throw Error(JJA_ERR_INTERNAL, "subtree staging exceeds shared memory");
      JJA_CUDA(cudaFuncSetAttribute(k_subtree<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      JJA_CUDA(cudaFuncSetAttribute(k_subtree<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    p->bwd_flow_items = p->up(S.bi_flow.data(), S.bi_flow.size());
    p->F.pack_meta = p->up(S.pack_meta.data(), S.pack_meta.size());
    p->F.pack_vals = p->up(S.pack_vals.data(), S.pack_vals.size());
    {
      // independent groups of problems for the step (level schedule only). Measured per step on
      // 128x128 arrays: W = 256 0.80 -> 0.70 ms with 2 groups; W = 512 1.36 -> 1.26 / 1.23 /
      // 1.23 ms with 2 / 3 / 4; W = 1024 2.61 -> 2.36 / 2.31 ms with 2 / 4; W = 64 (64x64) no gain
      const int chunks = (d->W + p->WB - 1) / p->WB;
      int ng = tu.groups ? tu.groups : (d->W >= kGroupsFromW ? std::max(2, std::min(4, d->W / kGroupW)) : 1);
      if (tu.schedule == 2 || tu.schedule == 3) ng = 1;
      ng = std::max(1, std::min(ng, chunks));
      if (ng > 1) {
        p->groups.resize(ng);
        JJA_CUDA(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming));
        for (int gi = 0; gi < ng; ++gi) {
          const int lo = (int)((int64_t)chunks * gi / ng) * p->WB;
          const int hi = std::min(d->W, (int)((int64_t)chunks * (gi + 1) / ng) * p->WB);
          const Schedule Sg = build_schedule(F, d->W, tu, lo, hi);
          if (Sg.n_levels != S.n_levels || Sg.subs.size() != S.subs.size())
            throw Error(JJA_ERR_INTERNAL, "group schedules differ in levels or subtrees");
          set_group(p->groups[gi], Sg, lo, hi - lo);
          if (gi > 0) JJA_CUDA(cudaStreamCreateWithFlags(&p->groups[gi].stream, cudaStreamNonBlocking));
          JJA_CUDA(cudaEventCreateWithFlags(&p->groups[gi].done, cudaEventDisableTiming));
        }
      }
    }
    {
      const int ns = S.ns;
      p->ns = ns;
      p->f_wait_on = p->up(S.fon.data(), S.fon.size());
      p->f_wait_count = p->up(S.fcnt.data(), S.fcnt.size());
      p->f_notify = p->up(S.fnot.data(), S.fnot.size());
      p->b_wait_on = p->up(S.bon.data(), S.bon.size());
      p->b_wait_count = p->up(S.bcnt.data(), S.bcnt.size());
      p->b_notify = p->up(S.bnot.data(), S.bnot.size());
      p->counters = p->up<unsigned>(nullptr, 2 * ((size_t)ns + 1));
      JJA_CUDA(cudaMemset(p->counters, 0, 2 * ((size_t)ns + 1) * sizeof(unsigned)));
      // device error flags: [0] a dataflow wait ran out, [1] a non-finite phase was produced
      p->flow_err = p->up<int>(nullptr, 2);
      JJA_CUDA(cudaMemset(p->flow_err, 0, 2 * sizeof(int)));
      p->t.nonfinite = p->flow_err + 1;
      int dev = 0, nsm = 0;
      JJA_CUDA(cudaGetDevice(&dev));
      JJA_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
      const void* kern[4][2] = {{(const void*)k_flow_sweep<2, false>, (const void*)k_flow_sweep<2, true>},
                                {(const void*)k_flow_sweep<4, false>, (const void*)k_flow_sweep<4, true>},
                                {(const void*)k_flow_sweep<8, false>, (const void*)k_flow_sweep<8, true>},
                                {(const void*)k_flow_sweep<1, false>, (const void*)k_flow_sweep<1, true>}};
      for (int v = 0; v < 4; ++v)
        for (int d = 0; d < 2; ++d) {
          int occ = 0;
          JJA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern[v][d], kWarpsPerBlock * 32, 0));
          p->flow_blocks[v][d] = std::max(1, occ) * nsm;
        }
      p->flow = (tu.schedule == 2) ? 1 : 0;
      // cooperative sweeps: blocks per launch within what can be resident at once (2 per SM at
      // most, fewer when the widest level has fewer items than the grid's warps, or as tuned)
      p->coop = (tu.schedule == 3) ? 1 : 0;
      if (p->coop) {
        p->coop_fwd_lp = p->up(S.fwd_ptr.data(), S.fwd_ptr.size());
        p->coop_bwd_lp = p->up(S.bwd_ptr.data(), S.bwd_ptr.size());
        p->coop_bar = p->up<unsigned>(nullptr, 2);
        JJA_CUDA(cudaMemset(p->coop_bar, 0, 2 * sizeof(unsigned)));
        for (char c : S.level_packed) p->coop_packs |= c != 0;
        int64_t widest[2] = {1, 1};
        for (int l = 0; l < S.n_levels; ++l) {
          widest[1] = std::max<int64_t>(widest[1], S.fwd_ptr[l + 1] - S.fwd_ptr[l]);
          widest[0] = std::max<int64_t>(widest[0], S.bwd_ptr[l + 1] - S.bwd_ptr[l]);
        }
        for (int fw = 0; fw < 2; ++fw)
          for (int pk = 0; pk < 2; ++pk) {
            const void* k = coop_kernel(fw ? p->rows_per_lane_fwd : p->rows_per_lane, fw != 0, pk != 0);
            int occ = 0;
            JJA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, kCoopThreads, 0));
            if (occ < 1) throw Error(JJA_ERR_CUDA, "cooperative sweep kernel cannot be resident");
            int64_t grid = (int64_t)std::min(occ, kCoopBlocksPerSM) * nsm;
            grid = std::min<int64_t>(grid, (widest[fw] + kCoopThreads / 32 - 1) / (kCoopThreads / 32));
            if (tu.coop_blocks) grid = std::min<int64_t>(grid, tu.coop_blocks);
            p->coop_grid[fw][pk] = (int)std::max<int64_t>(1, grid);
          }
      }
    }
    const size_t NfW = (size_t)Nf * d->W, NjW = (size_t)Nj * d->W;
    p->b = p->up<double>(nullptr, NfW);
    p->z = p->up<double>(nullptr, NfW);
    p->x = p->up<double>(nullptr, NfW);
    p->xj = p->up<double>(nullptr, NjW);
    p->isq = p->up<double>(nullptr, NjW);
    JJA_CUDA(cudaDeviceSynchronize());
    *out = p.release();
  });
}

void jja_plan_destroy(jja_plan* p) { delete p; }

int64_t jja_plan_device_bytes(const jja_plan* p) { return p ? p->bytes : 0; }

int jja_plan_set_fast_poisson(jja_plan* p, int mx, int my, const int32_t* grid_face, double kappa) {
  return guarded([&] {
    if (!p || !grid_face || mx < 1 || my < 1) throw Error(JJA_ERR_ARG, "jja_plan_set_fast_poisson: bad arguments");
    if ((int64_t)mx * my != p->Nf) throw Error(JJA_ERR_ARG, "jja_plan_set_fast_poisson: mx * my != Nf");
    if (!(kappa > 0.0)) throw Error(JJA_ERR_ARG, "jja_plan_set_fast_poisson: kappa must be positive");
    auto log2_of = [](int n) {   // log2(2 n) for n a power of two (n = m + 1), else -1
      if (n < 2 || (n & (n - 1))) return -1;
      int l = 1;
      while ((1 << l) < 2 * n) ++l;
      return l;
    };
    const int lgx = log2_of(mx + 1), lgy = log2_of(my + 1);
    if (lgx < 0 || lgy < 0 || mx + 1 > 1024 || my + 1 > 1024)
      throw Error(JJA_ERR_ARG, "jja_plan_set_fast_poisson: mx + 1 and my + 1 must be powers of two, at most 1024");
    std::vector<int32_t> gf((size_t)mx * my);
    std::vector<char> seen(p->Nf, 0);
    for (int64_t c = 0; c < (int64_t)mx * my; ++c) {
      const int f = grid_face[c];
      if (f < 0 || f >= p->Nf || seen[f]) throw Error(JJA_ERR_ARG, "jja_plan_set_fast_poisson: grid_face is not a permutation");
      seen[f] = 1;
      gf[c] = p->iperm_host[f];
    }
    const long double pi_l = 3.141592653589793238462643383279502884L;
    auto twiddles = [&](int m) {
      const int n = 2 * (m + 1);
      std::vector<double2> tw(n / 2);
      for (int k = 0; k < n / 2; ++k)
        tw[k] = make_double2((double)cosl(2 * pi_l * k / n), (double)-sinl(2 * pi_l * k / n));
      return tw;
    };
    auto eig = [&](int m) {
      std::vector<double> lam(m);
      for (int k = 0; k < m; ++k) lam[k] = (double)(2.0L - 2.0L * cosl(pi_l * (k + 1) / (m + 1)));
      return lam;
    };
    DstArgs& d = p->dst_args;
    d.mx = mx;
    d.my = my;
    d.lgx = lgx;
    d.lgy = lgy;
    d.grid_face = p->up(gf.data(), gf.size());
    const std::vector<double2> twx = twiddles(mx), twy = twiddles(my);
    d.twx = p->up(twx.data(), twx.size());
    d.twy = p->up(twy.data(), twy.size());
    const std::vector<double> lx = eig(mx), ly = eig(my);
    d.lamx = p->up(lx.data(), lx.size());
    d.lamy = p->up(ly.data(), ly.size());
    d.scale = (double)((4.0L / ((long double)(mx + 1) * (my + 1))) / kappa);
    d.t1 = p->up<double>(nullptr, (size_t)p->Nf * p->W);
    d.t2 = p->up<double>(nullptr, (size_t)p->Nf * p->W);
    const int smem_max = (int)(3 * 1024 * sizeof(double2) + 2 * 1023 * sizeof(double));
    JJA_CUDA(cudaFuncSetAttribute(k_dst_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
    JJA_CUDA(cudaFuncSetAttribute(k_dst_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
    // graphs captured before bake in the sweeps: drop them
    for (auto& g : p->graphs) cudaGraphExecDestroy(g.exec);
    for (auto& g : p->adj_graphs) cudaGraphExecDestroy(g.exec);
    p->graphs.clear();
    p->adj_graphs.clear();
    p->dst = 1;
  });
}

int jja_plan_test_wait_limit(jja_plan* p, void* stream) {
  return guarded([&] {
    if (!p) throw Error(JJA_ERR_ARG, "jja_plan_test_wait_limit: null plan");
    cudaStream_t st = (cudaStream_t)stream;
    if (p->coop) {
      // cooperative plan: a forward sweep whose barriers wait for one block more than the grid
      // has; each gives up after its bound, and the counters are reset by the next sweeps
      launch_coop<kDefaultRowsPerLane>(p, st, true, p->b, p->z, p->x, 1u);
      JJA_CUDA(cudaStreamSynchronize(st));
      JJA_CUDA(cudaMemsetAsync(p->coop_bar, 0, 2 * sizeof(unsigned), st));
      JJA_CUDA(cudaStreamSynchronize(st));
      return;
    }
    const std::vector<uint32_t> never((size_t)std::max(p->ns, 1), 0xffffffffu);
    uint32_t* d = nullptr;
    JJA_CUDA(cudaMalloc(&d, never.size() * sizeof(uint32_t)));
    const cudaError_t e1 = cudaMemcpy(d, never.data(), never.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e1 == cudaSuccess) {
      const int saved = p->flow;
      p->flow = 1;
      launch_zero_rows(p, st, true, p->z);
      launch_flow<kDefaultRowsPerLane>(p, st, true, p->b, p->z, p->x, d);
      p->flow = saved;
    }
    const cudaError_t e2 = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e1 != cudaSuccess) throw Error(JJA_ERR_CUDA, cudaGetErrorString(e1));
    if (e2 != cudaSuccess) throw Error(JJA_ERR_CUDA, cudaGetErrorString(e2));
  });
}

int jja_plan_check(jja_plan* p, int* flow_timeouts) {
  return guarded([&] {
    if (!p || !flow_timeouts) throw Error(JJA_ERR_ARG, "jja_plan_check: null argument");
    JJA_CUDA(cudaDeviceSynchronize());
    int h[2] = {0, 0};
    JJA_CUDA(cudaMemcpy(h, p->flow_err, 2 * sizeof(int), cudaMemcpyDeviceToHost));
    if (h[0] || h[1]) JJA_CUDA(cudaMemset(p->flow_err, 0, 2 * sizeof(int)));
    *flow_timeouts = h[0];
    if (h[1])
      throw Error(JJA_ERR_NONFINITE, "jja_plan_check: a time step produced a non-finite phase (NaN or inf) since the "
                                     "last check; the state and the outputs of those steps are invalid (check the "
                                     "inputs for NaN/inf, or a time step too large for the circuit)");
  });
}

int jja_solve(jja_plan* p, const double* b, double* x, void* stream) {
  return guarded([&] {
    if (!p || !b || !x) throw Error(JJA_ERR_ARG, "jja_solve: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t NfW = (int64_t)p->Nf * p->W;
    k_permute_rows<<<grid_for(NfW, 256), 256, 0, st>>>(b, p->b, p->perm, p->Nf, p->W, 1);
    g_launches++;
    launch_face_solve(p, st);
    k_permute_rows<<<grid_for(NfW, 256), 256, 0, st>>>(p->x, x, p->perm, p->Nf, p->W, 0);
    g_launches++;
    JJA_CUDA(cudaGetLastError());
  });
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// Allocation-free face-space solve (jja_solve_static). Its two work vectors live in this
// file-scope device array instead of memory from cudaMalloc: 32 MiB that every GPU which loads
// the library holds until the process exits. Host code must not use the array's name as a
// device address; the address is looked up once per device with cudaGetSymbolAddress.
// ------------------------------------------------------------------------------------------
namespace {

constexpr int64_t kStaticScratchDoubles = int64_t(4) << 20;   // 32 MiB
__device__ __align__(256) double g_static_scratch[kStaticScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
// the array's device address per device, and the CUDA context it was looked up in: a context
// that was destroyed and created again (cudaDeviceReset, a framework tearing down its primary
// context) loads the module anew, so the address is looked up again for a new context
struct StaticScratchSlot {
  void* ctx = nullptr;
  double* ptr = nullptr;
};
StaticScratchSlot g_static_slot[kMaxDevices];

// the calling thread's current CUDA context (driver entry point cuCtxGetCurrent, fetched through
// the runtime so the library needs no link-time dependency on the driver library)
void* current_context() {
  using CtxGetCurrent = int (*)(void**);
  static CtxGetCurrent fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<CtxGetCurrent>(f);
  }();
  if (!fn) throw Error(JJA_ERR_CUDA, "jja_solve_static: the driver entry point cuCtxGetCurrent is unavailable");
  void* ctx = nullptr;
  if (fn(&ctx) != 0 || !ctx) throw Error(JJA_ERR_CUDA, "jja_solve_static: no current CUDA context");
  return ctx;
}

double* static_scratch_for_current_device(cudaStream_t st) {
  int dev = 0;
  JJA_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) throw Error(JJA_ERR_ARG, "jja_solve_static: device index out of range");
  // a runtime call on the stream first: it binds the device's context to this thread
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  JJA_CUDA(cudaStreamIsCapturing(st, &cap));
  void* ctx = current_context();
  std::lock_guard<std::mutex> lock(g_static_mutex);
  StaticScratchSlot& slot = g_static_slot[dev];
  if (slot.ctx != ctx || !slot.ptr) {
    if (cap != cudaStreamCaptureStatusNone)
      throw Error(JJA_ERR_ARG, "jja_solve_static: the first call on a device (or after its context was re-created) "
                               "must come before any stream capture");
    void* ptr = nullptr;
    JJA_CUDA(cudaGetSymbolAddress(&ptr, g_static_scratch));
    slot.ctx = ctx;
    slot.ptr = static_cast<double*>(ptr);
  }
  return slot.ptr;
}

// the level sweeps of launch_levels with explicit work vectors
void launch_levels_into(jja_plan* p, cudaStream_t st, bool forward, double* b, double* z, double* x) {
  launch_zero_rows(p, st, forward, forward ? z : x);
  launch_sweep_any(p, st, forward, b, z, x);
}

}  // namespace

extern "C" {

int jja_solve_static(jja_plan* p, const double* b, double* x, void* stream) {
  return guarded([&] {
    if (!p || !b || !x) throw Error(JJA_ERR_ARG, "jja_solve_static: null argument");
    const int64_t NfW = (int64_t)p->Nf * p->W;
    if (2 * NfW > kStaticScratchDoubles)
      throw Error(JJA_ERR_ARG, "jja_solve_static: faces x problems = " + std::to_string(NfW) +
                                   " exceeds the static scratch limit of " +
                                   std::to_string(kStaticScratchDoubles / 2) + " (32 MiB for two work vectors)");
    cudaStream_t st = (cudaStream_t)stream;
    double* bx = static_scratch_for_current_device(st);   // permuted right-hand side, later the solution
    double* z = bx + NfW;                                // forward-substitution result
    // every element of both work vectors is written before it is read: nothing to clear
    k_permute_rows<<<grid_for(NfW, 256), 256, 0, st>>>(b, bx, p->perm, p->Nf, p->W, 1);
    g_launches++;
    launch_levels_into(p, st, true, bx, z, nullptr);
    launch_levels_into(p, st, false, nullptr, z, bx);
    k_permute_rows<<<grid_for(NfW, 256), 256, 0, st>>>(bx, x, p->perm, p->Nf, p->W, 0);
    g_launches++;
    JJA_CUDA(cudaGetLastError());
  });
}

// one backward-through-time step: a_n -> u = D a_n, b = A u, both sweeps, mu_n and accumulations
static void launch_adjoint_step(jja_plan* p, const AdjArgs& a, cudaStream_t st) {
  const int64_t NjW = (int64_t)p->Nj * p->W, NfW = (int64_t)p->Nf * p->W;
  k_adj_a<<<grid_for(NjW, 256), 256, 0, st>>>(a, p->t, p->xj);
  StepArgs s{};
  s.Nj = p->Nj; s.Nf = p->Nf; s.W = p->W; s.width = p->width; s.w0 = 0; s.wn = p->W; s.d_step = p->all.d_step;
  k_face_rhs<<<grid_for(NfW, 256), 256, 0, st>>>(s, p->t, p->xj, p->b);
  g_launches += 2;
  launch_face_solve(p, st);
  k_adj_mu<<<grid_for(NjW, 256), 256, 0, st>>>(a, p->t, p->xj, p->x);
  g_launches++;
}

int jja_adjoint_step(jja_plan* p, const jja_adjoint_args* g, void* stream) {
  return guarded([&] {
    if (!p || !g) throw Error(JJA_ERR_ARG, "jja_adjoint_step: null argument");
    if (p->width != 3) throw Error(JJA_ERR_ARG, "jja_adjoint_step: the adjoint supports stencil width 3 only");
    if (!g->th_m1 || !g->th_m2 || !g->mu_out || !g->cos_out || !g->usum || !g->musum || !g->gIc)
      throw Error(JJA_ERR_ARG, "jja_adjoint_step: missing buffer");
    if ((g->mu_p1 && !g->cos_p1) || (g->mu_p2 && !g->cos_p2))
      throw Error(JJA_ERR_ARG, "jja_adjoint_step: mu of a later step given without its cos(phi)");
    AdjArgs a{};
    a.Nj = p->Nj; a.W = p->W; a.G = g->G;
    a.th_m1 = g->th_m1; a.th_m2 = g->th_m2;
    a.mu_p1 = g->mu_p1; a.mu_p2 = g->mu_p2; a.cos_p1 = g->cos_p1; a.cos_p2 = g->cos_p2;
    a.mu_out = g->mu_out; a.cos_out = g->cos_out; a.usum = g->usum; a.musum = g->musum; a.gIc = g->gIc;
    launch_adjoint_step(p, a, (cudaStream_t)stream);
    JJA_CUDA(cudaGetLastError());
  });
}

int jja_adjoint_segment(jja_plan* p, const jja_adjoint_segment_args* g, void* stream) {
  return guarded([&] {
    if (!p || !g || !g->seg || g->L < 0 || g->s0 < 0 || g->s0 + g->L > g->Nt)
      throw Error(JJA_ERR_ARG, "jja_adjoint_segment: bad arguments");
    if (p->width != 3) throw Error(JJA_ERR_ARG, "jja_adjoint_segment: the adjoint supports stencil width 3 only");
    for (int k = 0; k < 3; ++k)
      if (!g->mu[k] || !g->cos[k]) throw Error(JJA_ERR_ARG, "jja_adjoint_segment: missing ring buffer");
    if (!g->usum || !g->musum || !g->gIc) throw Error(JJA_ERR_ARG, "jja_adjoint_segment: missing accumulator");
    const int64_t NjW = (int64_t)p->Nj * p->W;
    cudaStream_t st = (cudaStream_t)stream;
    auto walk = [&]() {
      for (int64_t i = g->L - 1; i >= 0; --i) {    // steps s0 + L - 1 down to s0
        const int64_t n = g->s0 + i;
        AdjArgs a{};
        a.Nj = p->Nj; a.W = p->W;
        const double* Gn = g->G ? g->G[i] : nullptr;
        a.G = jja_view{Gn, Gn ? p->W : 0, Gn ? 1 : 0, 0};
        a.th_m1 = g->seg + (i + 1) * NjW;          // theta_{n-1}
        a.th_m2 = g->seg + i * NjW;                // theta_{n-2}
        if (n + 1 < g->Nt) { a.mu_p1 = g->mu[(n + 1) % 3]; a.cos_p1 = g->cos[(n + 1) % 3]; }
        if (n + 2 < g->Nt) { a.mu_p2 = g->mu[(n + 2) % 3]; a.cos_p2 = g->cos[(n + 2) % 3]; }
        a.mu_out = g->mu[n % 3];
        a.cos_out = g->cos[n % 3];
        a.usum = g->usum; a.musum = g->musum; a.gIc = g->gIc;
        launch_adjoint_step(p, a, st);
      }
    };
    if (!g->use_graph || st == nullptr) {
      walk();
      JJA_CUDA(cudaGetLastError());
      return;
    }
    // The launches depend on the step only through step % 3, the distance to the end of the
    // run (missing later steps) and the loss-weight pointers: segments that agree on those and
    // on the buffers share one captured graph.
    std::vector<uint64_t> key = {(uint64_t)g->seg, (uint64_t)g->L, (uint64_t)(g->s0 % 3),
                                 (uint64_t)std::min<int64_t>(g->Nt - g->s0 - g->L, 3), (uint64_t)st,
                                 (uint64_t)g->usum, (uint64_t)g->musum, (uint64_t)g->gIc};
    for (int k = 0; k < 3; ++k) {
      key.push_back((uint64_t)g->mu[k]);
      key.push_back((uint64_t)g->cos[k]);
    }
    for (int64_t i = 0; i < g->L; ++i) key.push_back((uint64_t)(g->G ? g->G[i] : nullptr));
    cudaGraphExec_t exec = nullptr;
    for (size_t k = 0; k < p->adj_graphs.size(); ++k)
      if (p->adj_graphs[k].key == key) { exec = p->adj_graphs[k].exec; break; }
    if (!exec) {
      if (p->adj_graphs.size() >= jja_plan::kMaxGraphs) {
        cudaGraphExecDestroy(p->adj_graphs.front().exec);
        p->adj_graphs.erase(p->adj_graphs.begin());
      }
      cudaGraph_t graph;
      JJA_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      walk();
      JJA_CUDA(cudaStreamEndCapture(st, &graph));
      const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) throw Error(JJA_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
      p->adj_graphs.push_back({key, exec});
    }
    JJA_CUDA(cudaGraphLaunch(exec, st));
    JJA_CUDA(cudaGetLastError());
  });
}

int jja_adjoint_flux(jja_plan* p, const double* usum, double* gf, void* stream) {
  return guarded([&] {
    if (!p || !usum || !gf) throw Error(JJA_ERR_ARG, "jja_adjoint_flux: null argument");
    cudaStream_t st = (cudaStream_t)stream;
    const int64_t NfW = (int64_t)p->Nf * p->W;
    StepArgs s{};
    s.Nj = p->Nj; s.Nf = p->Nf; s.W = p->W; s.width = p->width; s.w0 = 0; s.wn = p->W; s.d_step = p->all.d_step;
    k_face_rhs<<<grid_for(NfW, 256), 256, 0, st>>>(s, p->t, usum, p->b);
    g_launches++;
    launch_face_solve(p, st);
    k_unpermute_scaled<<<grid_for(NfW, 256), 256, 0, st>>>(p->x, gf, p->perm, p->Nf, p->W, -kTwoPi);
    g_launches++;
    JJA_CUDA(cudaGetLastError());
  });
}

int jja_vortex(jja_plan* p, const double* theta, int64_t n_steps, int32_t* n_out, uint64_t* flow, void* stream) {
  return guarded([&] {
    if (!p || !theta || n_steps < 0) throw Error(JJA_ERR_ARG, "jja_vortex: bad arguments");
    if (!n_steps || (!n_out && !flow)) return;
    cudaStream_t st = (cudaStream_t)stream;
    k_vortex<<<grid_for((int64_t)p->Nf * p->W, 256), 256, 0, st>>>(theta, n_steps, p->Nj, p->Nf, p->W, p->t, n_out,
                                                                    reinterpret_cast<unsigned long long*>(flow));
    g_launches++;
    JJA_CUDA(cudaGetLastError());
  });
}

int jja_eval_sin(jja_plan* p, const double* x, double* out, int64_t n, void* stream) {
  return guarded([&] {
    if (!p || !x || !out || n < 0) throw Error(JJA_ERR_ARG, "jja_eval_sin: bad arguments");
    if (n == 0) return;
    k_eval_sin<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(x, out, n, p->t.sincos);
    g_launches++;
    JJA_CUDA(cudaGetLastError());
  });
}

int jja_sin_host(const double* x, double* s, double* c, int64_t n) {
  return guarded([&] {
    if (!x || n < 0 || (!s && !c)) throw Error(JJA_ERR_ARG, "jja_sin_host: bad arguments");
    static const std::vector<longlong2> tab = build_sin_table();
    for (int64_t i = 0; i < n; ++i) {
      double sv, cv;
      fast_sincos(x[i], tab.data(), sv, cv);
      if (s) s[i] = c ? sv : fast_sin(x[i], tab.data());
      if (c) c[i] = cv;
    }
  });
}

int jja_run(jja_plan* p, jja_state* s, int nsteps, const int64_t* th_slot, const int64_t* I_slot, int use_graph,
            void* stream) {
  return guarded([&] {
    if (!p || !s || nsteps < 0) throw Error(JJA_ERR_ARG, "jja_run: bad arguments");
    for (int k = 0; k < p->width - 1; ++k)
      if (!s->hist[k]) throw Error(JJA_ERR_ARG, "jja_run: missing history buffer");
    if (s->noise_mode == JJA_NOISE_BUFFER && !s->noise) throw Error(JJA_ERR_ARG, "jja_run: noise buffer missing");
    if (s->store_all && (th_slot || I_slot))
      throw Error(JJA_ERR_ARG, "jja_run: store_all replaces th_slot / I_slot (pass NULL)");
    if (nsteps == 0) return;
    check_window(s, nsteps, "jja_run");
    cudaStream_t st = (cudaStream_t)stream;
    const std::vector<Group*> gs = step_groups(p);
    set_counters(p, s, st);
    launch_scale_sources(p, s, st);
    fork_groups(p, st);
    for (Group* g : gs) {
      StepArgs a = make_args(p, s, *g);
      launch_junction(p, a, stream_of(*g, st));
    }
    join_groups(p, st);
    const int period = p->width - 1;  // history rotation period
    int i = 0;
    while (i < nsteps) {
      // a run of steps that store nothing (or, with store_all, whose slots the device derives
      // from the step counter) can be replayed from captured graphs; the call's last step
      // stays out of them (it runs unfused: the look-ahead q it would evaluate belongs to a step
      // outside this call, whose sources may lie outside the source window)
      int run = 0;
      while (i + run < nsteps && (!th_slot || th_slot[i + run] < 0) && (!I_slot || I_slot[i + run] < 0)) ++run;
      const int graphable = (i + run == nsteps) ? run - 1 : run;
      // capture needs a non-default stream; the per-step noise buffer is refilled by the host.
      // Graphs hold 16, 8, 4, 2 or 1 rotation periods of steps (pointers return to their places
      // after each), taken greedily, so short runs replay graphs too and at most one period of
      // steps runs eagerly
      if (use_graph && st != nullptr && graphable >= period && s->noise_mode != JJA_NOISE_BUFFER) {
        int done = 0;
        for (int mult = 16; mult >= 1; mult >>= 1) {
          const int G = mult * period;
          if (graphable - done < G) continue;
          cudaGraphExec_t exec = graph_for(p, s, st, G);
          const int reps = (graphable - done) / G;
          for (int r = 0; r < reps; ++r) JJA_CUDA(cudaGraphLaunch(exec, st));
          done += reps * G;
        }
        i += done;
        run -= done;
      }
      const int eager = (i < nsteps) ? std::max(run, 1) : 0;
      if (eager > 0 && i < nsteps) {
        fork_groups(p, st);
        for (int q = 0; q < eager && i < nsteps; ++q, ++i) {
          for (Group* g : gs) {
            StepArgs a = make_args(p, s, *g);
            a.hout = s->hist[period - 1];
            a.th_slot = th_slot ? th_slot[i] : -1;
            a.I_slot = I_slot ? I_slot[i] : -1;
            launch_step(p, *g, a, stream_of(*g, st), i + 1 < nsteps);
          }
          rotate(s, p->width);
        }
        join_groups(p, st);
      }
    }
    JJA_CUDA(cudaGetLastError());
    s->step += nsteps;
  });
}

int jja_run_timed(jja_plan* p, jja_state* s, int nsteps, double* stage_ms, void* stream) {
  return guarded([&] {
    if (!p || !s || nsteps <= 0 || !stage_ms) throw Error(JJA_ERR_ARG, "jja_run_timed: bad arguments");
    if (s->noise_mode == JJA_NOISE_BUFFER) throw Error(JJA_ERR_ARG, "jja_run_timed: host noise buffer not supported");
    check_window(s, nsteps, "jja_run_timed");
    cudaStream_t st = (cudaStream_t)stream;
    set_counters(p, s, st);
    std::vector<cudaEvent_t> ev(1 + 5 * (size_t)nsteps);
    for (auto& e : ev) JJA_CUDA(cudaEventCreate(&e));
    JJA_CUDA(cudaEventRecord(ev[0], st));
    launch_scale_sources(p, s, st);
    const std::vector<Group*> gs = step_groups(p);
    fork_groups(p, st);
    for (Group* g : gs) {
      StepArgs a = make_args(p, s, *g);
      launch_junction(p, a, stream_of(*g, st));
    }
    join_groups(p, st);
    // stage by stage: the groups run each stage concurrently on their streams and join back
    // into the caller's stream at every stage boundary, where the events are recorded
    const int period = p->width - 1;
    for (int i = 0; i < nsteps; ++i) {
      cudaEvent_t* e = ev.data() + 1 + 5 * (size_t)i;
      std::vector<StepArgs> args;
      for (Group* g : gs) {
        args.push_back(make_args(p, s, *g));
        args.back().hout = s->hist[period - 1];
        args.back().th_slot = args.back().I_slot = -1;
      }
      auto stage = [&](int k, auto&& fn) {
        fork_groups(p, st);
        for (size_t q = 0; q < gs.size(); ++q) fn(q, stream_of(*gs[q], st));
        join_groups(p, st);
        JJA_CUDA(cudaEventRecord(e[k], st));
      };
      JJA_CUDA(cudaEventRecord(e[0], st));
      stage(1, [&](size_t q, cudaStream_t gst) {
        launch(p->pdl, k_face_rhs, grid_for((int64_t)p->Nf * gs[q]->wn, 256), 256, gst, args[q], p->t,
               (const double*)p->xj, p->b);
      });
      // (a fast Poisson plan solves in the "forward" stage; its "backward" stage is empty)
      stage(2, [&](size_t q, cudaStream_t gst) {
        if (p->dst) launch_face_solve(p, *gs[q], gst);
        else launch_levels(p, *gs[q], gst, true);
      });
      stage(3, [&](size_t q, cudaStream_t gst) {
        if (!p->dst) launch_levels(p, *gs[q], gst, false);
      });
      stage(4, [&](size_t q, cudaStream_t gst) {
        const int64_t nj = (int64_t)p->Nj * gs[q]->wn;
        if (i + 1 < nsteps)
          launch(p->pdl, k_update<true>, grid_for(nj, 256), 256, gst, args[q], p->t, p->xj, (const double*)p->x);
        else
          launch(p->pdl, k_update<false>, grid_for(nj, 256), 256, gst, args[q], p->t, p->xj, (const double*)p->x);
      });
      rotate(s, p->width);
    }
    JJA_CUDA(cudaEventSynchronize(ev.back()));
    for (int k = 0; k < 6; ++k) stage_ms[k] = 0.0;
    float ms = 0.f;
    JJA_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    stage_ms[0] = ms;  // first junction evaluation
    for (int i = 0; i < nsteps; ++i) {
      const cudaEvent_t* e = ev.data() + 1 + 5 * (size_t)i;
      for (int k = 0; k < 4; ++k) {
        JJA_CUDA(cudaEventElapsedTime(&ms, e[k], e[k + 1]));
        stage_ms[1 + k] += ms;
      }
    }
    JJA_CUDA(cudaEventElapsedTime(&ms, ev.front(), ev.back()));
    stage_ms[5] = ms;
    for (auto& e : ev) cudaEventDestroy(e);
    s->step += nsteps;
  });
}

}  // extern "C"
#include "jja_static.cuh"
