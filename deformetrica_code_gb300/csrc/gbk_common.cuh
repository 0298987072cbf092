// Device-side building blocks shared by every Gaussian kernel-sum kernel.
//
// Precision model. The bulk arithmetic runs in FP32 on *pairs of targets* packed in float2 and
// issued as Blackwell's packed FP32 instructions (FADD2/FMUL2/FFMA2 through the __fadd2_rn /
// __fmul2_rn / __ffma2_rn builtins), so one instruction advances two kernel pairs. exp is
// evaluated on the MUFU unit as 2^(r2 * c) with c = -log2(e)/sigma^2 (ex2.approx.ftz.f32): the
// identity e^-a = 2^(-a log2 e). Each target accumulates a short run of sources in plain FP32 and
// then folds the run into a (sum, compensation) pair with an error-free TwoSum, so the
// compensation costs a few instructions per run rather than per pair. The FP64 mode uses the same
// kernels with double lanes, libm-equivalent exp() and no compensation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include <utility>

namespace gbk {

// ---------------------------------------------------------------------------------------------
// Programmatic dependent launch. A kernel launched through launch() below may be placed on the
// SMs while the previous kernel of its stream is still running, so its launch latency and CTA
// placement overlap the predecessor's tail; this matters for the deformation loops' hundreds of
// small dependent launches inside one CUDA graph. Every kernel of the library begins with
// pdl_entry(): griddepcontrol.wait blocks until the predecessor grid has completed and its memory
// is visible, so nothing is read or written earlier than in plain stream order, and then
// griddepcontrol.launch_dependents lets the next kernel be placed. Launched without the attribute
// (<<<>>>, or GBK_PDL=0 in the environment), both instructions do nothing.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void pdl_entry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Programmatic launches are on unless GBK_PDL=0 (read once per process).
inline bool pdl_enabled() {
  static const bool on = [] {
    const char *e = getenv("GBK_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

// kern<<<grid, block, smem, st>>>(args...) with programmatic stream serialisation allowed.
template <typename... KArgs, typename... Args>
inline cudaError_t launch(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                          Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// ---------------------------------------------------------------------------------------------
// Index checks of a bounds-checked build (-DGBK_BOUNDS_CHECK=1; compiled out otherwise): an index
// outside [0, n) sets bit 1 of the launch's status word (gbk_synchronize reports GBK_ERR_BOUNDS) and
// is clamped into the array, so a checked kernel never reads or writes outside its arrays.
// ---------------------------------------------------------------------------------------------
#ifndef GBK_BOUNDS_CHECK
#define GBK_BOUNDS_CHECK 0
#endif
__device__ __forceinline__ long checked_index(long i, long n, unsigned *status) {
#if GBK_BOUNDS_CHECK
  if (i < 0 || i >= n) {
    if (status) atomicOr(status, 2u);
    return i < 0 || n <= 0 ? 0 : n - 1;
  }
#else
  (void)n;
  (void)status;
#endif
  return i;
}

// ---------------------------------------------------------------------------------------------
// Lane types: Lane<float> carries two targets (float2, packed FFMA2), Lane<f32s> one target in
// scalar FP32, Lane<double> one target in FP64. Packed FFMA2 halves issue slots, but with three
// distinct register operands per instruction it measured ~68% of the FP32 lane peak on GB300
// (operand bandwidth) against ~78% for scalar FFMA, so both FP32 forms are kept.
// ---------------------------------------------------------------------------------------------
struct f32s {};  // tag: scalar FP32 lanes
// Tag: packed FP32 lanes (as float) with two-float coordinates. Each centred, scaled coordinate is
// kept as hi + lo, hi = fl32(c) and lo = fl32(c - hi), and a pair's difference is formed as
// (x_hi - y_hi) + (x_lo - y_lo): its error is ~2u |x - y| instead of ~u (|x| + |y|), so accuracy no
// longer depends on how far the CTA's points spread from its centre (caller order on data spread
// wide relative to sigma). Costs 2 packed adds per coordinate per pair.
struct f32w {};
// Tag: packed FP32 lanes (as float) whose source tiles are staged by bulk asynchronous copies
// (cp.async.bulk into a double-buffered shared area, completion tracked by mbarriers) when the
// launch's sources are the library's own chunk-padded sorted copies (PairArgs::bulk); otherwise the
// kernel stages with ordinary loads. Same arithmetic, same bits as float.
struct f32b {};

template <typename T>
struct Lane;

template <>
struct Lane<float> {
  typedef float2 V;
  static constexpr int kWidth = 2;
  __device__ __forceinline__ static V add(V a, V b) { return __fadd2_rn(a, b); }
  // a - b as one packed FMA with -1 (exact product, single rounding): there is no packed FSUB.
  __device__ __forceinline__ static V sub(V a, V b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
  __device__ __forceinline__ static V mul(V a, V b) { return __fmul2_rn(a, b); }
  __device__ __forceinline__ static V fma(V a, V b, V c) { return __ffma2_rn(a, b, c); }
  __device__ __forceinline__ static V zero() { return make_float2(0.f, 0.f); }
  __device__ __forceinline__ static V splat(float s) { return make_float2(s, s); }
  // K = 2^(-r2') per lane on the MUFU unit. Coordinates are pre-scaled by sqrt(log2 e)/sigma,
  // so r2' = |x' - y'|^2 = |x - y|^2 log2(e) / sigma^2 and 2^(-r2') = exp(-|x - y|^2 / sigma^2).
  // Results below 2^-126 flush to zero.
  __device__ __forceinline__ static V kexp(V r2, V) {
    float a, b;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(a) : "f"(-r2.x));
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(b) : "f"(-r2.y));
    return make_float2(a, b);
  }
  __device__ __forceinline__ static float get(V v, int l) { return l == 0 ? v.x : v.y; }
  __device__ __forceinline__ static V make(float a, float b) { return make_float2(a, b); }
};

template <>
struct Lane<f32w> : Lane<float> {};
template <>
struct Lane<f32b> : Lane<float> {};

template <>
struct Lane<f32s> {
  typedef float V;
  static constexpr int kWidth = 1;
  __device__ __forceinline__ static V add(V a, V b) { return __fadd_rn(a, b); }
  __device__ __forceinline__ static V sub(V a, V b) { return __fsub_rn(a, b); }
  __device__ __forceinline__ static V mul(V a, V b) { return __fmul_rn(a, b); }
  __device__ __forceinline__ static V fma(V a, V b, V c) { return __fmaf_rn(a, b, c); }
  __device__ __forceinline__ static V zero() { return 0.f; }
  __device__ __forceinline__ static V splat(float s) { return s; }
  __device__ __forceinline__ static V kexp(V r2, V) {
    float a;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(a) : "f"(-r2));
    return a;
  }
  __device__ __forceinline__ static float get(V v, int) { return v; }
};

template <>
struct Lane<double> {
  typedef double V;
  static constexpr int kWidth = 1;
  __device__ __forceinline__ static V add(V a, V b) { return __dadd_rn(a, b); }
  __device__ __forceinline__ static V sub(V a, V b) { return __dsub_rn(a, b); }
  __device__ __forceinline__ static V mul(V a, V b) { return __dmul_rn(a, b); }
  __device__ __forceinline__ static V fma(V a, V b, V c) { return __fma_rn(a, b, c); }
  __device__ __forceinline__ static V zero() { return 0.0; }
  __device__ __forceinline__ static V splat(double s) { return s; }
  // FP64 mode: unscaled coordinates, K = exp(r2 * (-1/sigma^2)) with the CUDA math library.
  __device__ __forceinline__ static V kexp(V r2, V cx) { return exp(r2 * cx); }
  __device__ __forceinline__ static double get(V v, int) { return v; }
};

// Source values are stored in shared memory already broadcast to the lane type.
template <typename T>
struct SrcVal;
template <>
struct SrcVal<float> {
  __device__ __forceinline__ static float2 make(double v) {
    float f = (float)v;
    return make_float2(f, f);
  }
  __device__ __forceinline__ static float2 make(float f) { return make_float2(f, f); }
};
template <>
struct SrcVal<f32w> : SrcVal<float> {};
template <>
struct SrcVal<f32b> : SrcVal<float> {};
template <>
struct SrcVal<f32s> {
  __device__ __forceinline__ static float make(double v) { return (float)v; }
  __device__ __forceinline__ static float make(float v) { return v; }
};
template <>
struct SrcVal<double> {
  __device__ __forceinline__ static double make(double v) { return v; }
};

// ---------------------------------------------------------------------------------------------
// Compensated accumulation: (sum, comp) += run, with Knuth's error-free TwoSum.
// ---------------------------------------------------------------------------------------------
template <typename T>
struct Comp {
  typedef typename Lane<T>::V V;
  __device__ __forceinline__ static void fold(V &sum, V &comp, V run) {
    typedef Lane<T> L;
    V s = L::add(sum, run);
    V bb = L::sub(s, sum);
    V err = L::add(L::sub(sum, L::sub(s, bb)), L::sub(run, bb));
    comp = L::add(comp, err);
    sum = s;
  }
};
template <>
struct Comp<f32w> : Comp<float> {};
template <>
struct Comp<f32b> : Comp<float> {};
template <>
struct Comp<f32s> {
  __device__ __forceinline__ static void fold(float &sum, float &comp, float run) {
    float s = __fadd_rn(sum, run);
    float bb = __fsub_rn(s, sum);
    float err = __fadd_rn(__fsub_rn(sum, __fsub_rn(s, bb)), __fsub_rn(run, bb));
    comp = __fadd_rn(comp, err);
    sum = s;
  }
};
template <>
struct Comp<double> {
  __device__ __forceinline__ static void fold(double &sum, double &, double run) { sum += run; }
};

// Coordinate pre-scale of each lane type: FP32 works on x' = x sqrt(log2 e) / sigma (scaled in
// FP64 before rounding, so x' keeps the relative precision of a rounded x); FP64 keeps x.
template <typename T>
__host__ __device__ inline double coord_scale(double sigma);
template <>
__host__ __device__ inline double coord_scale<float>(double sigma) {
  return 1.2011224087864498 / sigma;  // sqrt(log2(e)) / sigma
}
template <>
__host__ __device__ inline double coord_scale<f32s>(double sigma) {
  return 1.2011224087864498 / sigma;
}
template <>
__host__ __device__ inline double coord_scale<f32w>(double sigma) {
  return 1.2011224087864498 / sigma;
}
template <>
__host__ __device__ inline double coord_scale<f32b>(double sigma) {
  return 1.2011224087864498 / sigma;
}
template <>
__host__ __device__ inline double coord_scale<double>(double) {
  return 1.0;
}
// Scale of r2 inside kexp (FP64 only): -1/sigma^2.
template <typename T>
__host__ __device__ inline typename Lane<T>::V exp_arg_scale(double sigma) {
  return (typename Lane<T>::V)(-1.0 / (sigma * sigma));
}
template <>
__host__ __device__ inline float2 exp_arg_scale<float>(double sigma) {
  return float2{0.f, 0.f};  // unused: FP32 lanes work on pre-scaled coordinates
}
template <>
__host__ __device__ inline float2 exp_arg_scale<f32w>(double sigma) {
  return float2{0.f, 0.f};
}
template <>
__host__ __device__ inline float2 exp_arg_scale<f32b>(double sigma) {
  return float2{0.f, 0.f};
}

// Squared distance (input units) beyond which the lane type's kernel value is exactly zero, with
// margin. FP32 lanes evaluate ex2.approx.ftz(-r2) on coordinates scaled by coord_scale: for
// r2 >= 127 the result is subnormal and flushed to +0, and 130 leaves room for the FP32 rounding
// of r2. FP64 lanes evaluate exp(-|dx|^2 / sigma^2), which is below half the smallest subnormal
// (exp(-745.13)) and rounds to zero for arguments under -800.
template <typename T>
inline double prune_dist2(double sigma) {
  const double s = coord_scale<T>(sigma);
  return 130.0 / (s * s);
}
template <>
inline double prune_dist2<double>(double sigma) {
  return 800.0 * sigma * sigma;
}

// ---------------------------------------------------------------------------------------------
// Bulk asynchronous copies global -> shared (cp.async.bulk) completed on an mbarrier in shared
// memory. Addresses must be 16-byte aligned and sizes multiples of 16 bytes; an mbarrier phase
// takes at most 2^20 - 1 bytes of transactions.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
// makes the initialised barriers visible to the asynchronous proxy
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// one arrival that also announces `bytes` of transactions for the current phase
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Waits for the phase of `parity` to complete for at most ~2^31 SM clock cycles (about one second);
// false if it did not.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > (1LL << 31)) return false;
  return true;
}
// orders this thread's earlier generic-proxy accesses of shared memory before later asynchronous
// copies into it (the buffer being refilled was read by ordinary loads)
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}

}  // namespace gbk
