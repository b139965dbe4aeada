// device_common.cuh -- device-side building blocks shared by the setpts,
// spread, interp and deconvolution kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nufft_types.h"

namespace cfg {

// ---- exact-rounding arithmetic (never contracted into FMAs) --------------
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float floor_t(float a) { return floorf(a); }
__device__ __forceinline__ double floor_t(double a) { return floor(a); }
__device__ __forceinline__ float ceil_t(float a) { return ceilf(a); }
__device__ __forceinline__ double ceil_t(double a) { return ceil(a); }

// pi rounded to the plan precision: the fold branch compares against it, as
// the reference's RESCALE macro does with PI = (FLT)M_PI
// (contrib/spreadinterp.h:36-38, contrib/utils.h:21).
template <typename T> __device__ __forceinline__ T pi_t();
template <> __device__ __forceinline__ float pi_t<float>() { return 3.14159265358979323846f; }
template <> __device__ __forceinline__ double pi_t<double>() { return 3.14159265358979323846; }

// Fine-grid placement of one coordinate.  The reference computes the
// rescaled position t = (x/(2 pi) + shift) * nf (shift 0.5, or 1.5 / -0.5 to
// fold [-3pi,-pi) and [pi,3pi)), first tap i0 = ceil(t - ns/2) and tap
// offsets i0 + j - t (src/2d/spreadinterp2d.cu:22-33).  Here t is carried as
// an unevaluated sum t_hi + t_lo (error-free product and sum), so the stored
// offset d = i0 - t + ns/2 in [0,1) keeps ~1 ulp of [0,1) even in FP32,
// where a rounded t in [0, nf) would lose log2(nf) bits.
//   i0 is returned wrapped into [0, nf); tap j sits at (i0 + j) mod nf with
//   kernel argument d - ns/2 + j.
template <typename T>
__device__ __forceinline__ void place_coord(T x, const AxisMap<T>& a, int& i0, T& d) {
  const T pi = pi_t<T>();
  T o = (x < -pi) ? a.o_lo : ((x >= pi) ? a.o_hi : a.o_mid);
  T p_hi = mul_rn(x, a.s_hi);
  T p_err = fma_rn(x, a.s_hi, -p_hi);
  T p_lo = fma_rn(x, a.s_lo, p_err);
  T t_hi = add_rn(p_hi, o);
  T bb = sub_rn(t_hi, p_hi);
  T err = add_rn(sub_rn(p_hi, sub_rn(t_hi, bb)), sub_rn(o, bb));
  T t_lo = add_rn(err, p_lo);
  T fl = floor_t(t_hi);
  T g = add_rn(sub_rn(t_hi, fl), t_lo);   // fractional position ~[0,1)
  T gg = sub_rn(g, a.half_frac);          // minus the fractional part of ns/2
  T cg = ceil_t(gg);
  d = sub_rn(cg, gg);                     // in [0, 1)
  int i = (int)fl + (int)cg - a.half_int;
  if (i < 0) i += a.nf;
  if (i >= a.nf) i -= a.nf;
  // points outside [-3pi,3pi) (or non-finite ones) still land in [0, nf):
  // every grid access stays in bounds whatever the input
  if (i < 0 || i >= a.nf) i = ((i % a.nf) + a.nf) % a.nf;
  i0 = i;
}

// ---- ES kernel values -----------------------------------------------------
// phi = exp(beta*sqrt(1 - z)) for z = c x^2 < 1, else 0; evaluated without a
// branch (the square root of a clamped argument, then a select).
//
// FP32 uses sqrt(1-z) - 1 = -z / (1 + sqrt(1-z)):
//   phi = e^beta * 2^(-(beta log2 e) z / (1 + sqrt(1 - z))).
// The exponent is near 0 where phi is large and large only where phi is
// small, so the PTX approximations of sqrt, 1/x and 2^x (each within a few
// ulps) keep a few-ulp error relative to the peak everywhere; the direct
// form expf(beta * sqrtf(1 - z)) loses about beta ulps at the peak to the
// rounding of its argument.  e_beta = e^beta and bl2e = beta log2 e are
// rounded once on the host.  FP64 uses the direct form.
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float es_value_fast(float z, float e_beta, float bl2e) {
  const float s = sqrt_approx(fmaxf(1.0f - z, 0.0f));
  const float v = ex2_approx(-bl2e * z * rcp_approx(1.0f + s)) * e_beta;
  return z < 1.0f ? v : 0.0f;
}

__device__ __forceinline__ double es_value(double z, double beta) {
  const double e = exp(beta * sqrt(fmax(1.0 - z, 0.0)));
  return z < 1.0 ? e : 0.0;
}

// The kernel value the spread/interp kernels use.  (Defined after the
// evaluators it calls: the names in a template are bound where it is
// defined.)
template <typename T>
__device__ __forceinline__ T es_eval(T z, const KernelCoeffs<T>& kc) {
  if constexpr (sizeof(T) == 4) return es_value_fast(z, kc.e_beta, kc.bl2e);
  else return es_value(z, kc.beta);
}

// ker[j] = phi(d - ns/2 + j), j = 0..NS-1, phi(x) = exp(beta*sqrt(1-c x^2))
// for |x| < ns/2 and 0 outside (src/cuspreadinterp.h:6-40).  With
// kc.horner set the values come from the plan's fitted piecewise
// polynomials in z = 2d - 1 (coefficient k of tap j at coef[k*NS + j],
// highest degree first, HDEG+1 rows).
// FP32 row of ES values two taps at a time: es_value_fast's steps on each
// tap, the plain multiplies and adds as packed f32x2 instructions (each half
// an IEEE operation; 1 - z is rounded after z, where the compiler may fuse
// the scalar form into one fma, so values can differ from it by an ulp).
template <int NS>
__device__ __forceinline__ void es_row_f32x2(float d, const KernelCoeffs<float>& kc, float* ker) {
  const float x0 = d - 0.5f * NS;
  const float2 c2 = make_float2(kc.c, kc.c), one = make_float2(1.0f, 1.0f);
  const float2 mone = make_float2(-1.0f, -1.0f), mb = make_float2(-kc.bl2e, -kc.bl2e);
  const float2 eb = make_float2(kc.e_beta, kc.e_beta);
#pragma unroll
  for (int j = 0; j + 1 < NS; j += 2) {
    const float2 x = __fadd2_rn(make_float2(x0, x0), make_float2(float(j), float(j + 1)));
    const float2 z = __fmul2_rn(__fmul2_rn(c2, x), x);
    const float2 u = __ffma2_rn(z, mone, one);  // 1 - z
    const float2 s = make_float2(sqrt_approx(fmaxf(u.x, 0.0f)), sqrt_approx(fmaxf(u.y, 0.0f)));
    const float2 q = __fadd2_rn(one, s);
    const float2 e = __fmul2_rn(__fmul2_rn(mb, z), make_float2(rcp_approx(q.x), rcp_approx(q.y)));
    const float2 v = __fmul2_rn(make_float2(ex2_approx(e.x), ex2_approx(e.y)), eb);
    ker[j] = z.x < 1.0f ? v.x : 0.0f;
    ker[j + 1] = z.y < 1.0f ? v.y : 0.0f;
  }
  if (NS & 1) ker[NS - 1] = es_value_fast(kc.c * (x0 + float(NS - 1)) * (x0 + float(NS - 1)), kc.e_beta, kc.bl2e);
}

template <typename T, int NS, int HDEG>
__device__ __forceinline__ void kernel_row(T d, const KernelCoeffs<T>& kc, T* ker) {
  if (kc.horner) {
    const T z = T(2) * d - T(1);
#pragma unroll
    for (int j = 0; j < NS; ++j) ker[j] = kc.coef[j];
#pragma unroll
    for (int k = 1; k <= HDEG; ++k) {
#pragma unroll
      for (int j = 0; j < NS; ++j) ker[j] = fma_rn(ker[j], z, kc.coef[k * NS + j]);
    }
  } else if constexpr (sizeof(T) == 4) {
    es_row_f32x2<NS>(d, kc, ker);
  } else {
    const T x0 = d - T(0.5) * T(NS);
#pragma unroll
    for (int j = 0; j < NS; ++j) {
      const T x = x0 + T(j);
      ker[j] = es_eval(kc.c * x * x, kc);
    }
  }
}

// One kernel value phi(d - ns/2 + j) for a runtime tap index j (used along
// the outermost axis of 3D loops, which are not unrolled).
template <typename T, int NS, int HDEG>
__device__ __forceinline__ T kernel_tap(T d, int j, const KernelCoeffs<T>& kc) {
  if (kc.horner) {
    const T z = T(2) * d - T(1);
    T v = __ldg(kc.coef_g + j);
#pragma unroll
    for (int k = 1; k <= HDEG; ++k) v = fma_rn(v, z, __ldg(kc.coef_g + k * NS + j));
    return v;
  }
  const T x = d - T(0.5) * T(NS) + T(j);
  return es_eval(kc.c * x * x, kc);
}

// ---- double-float arithmetic (FP64 plans without FP64 units) -------------
// A value is an unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2):
// ~48 bits of mantissa.  Error-free transformations: two_sum (Knuth) and
// the FMA product error; every step rounds explicitly, so the compiler never
// contracts or reassociates them.
struct DF {
  float h, l;
};
__device__ __forceinline__ DF df_from(double v) {
  DF r;
  r.h = __double2float_rn(v);
  r.l = __double2float_rn(v - (double)r.h);
  return r;
}
__device__ __forceinline__ double df_to(DF a) { return (double)a.h + (double)a.l; }
// s + e = a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ DF df_renorm(float s, float e) {
  DF r;
  r.h = __fadd_rn(s, e);
  r.l = __fsub_rn(e, __fsub_rn(r.h, s));
  return r;
}
__device__ __forceinline__ DF df_add(DF a, DF b) {
  float s, e;
  two_sum(a.h, b.h, s, e);
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  return df_renorm(s, e);
}
// a * b to ~2^-47 relative (the lo*lo term is dropped)
__device__ __forceinline__ DF df_mul(DF a, DF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return df_renorm(p, e);
}
// acc + a * b
__device__ __forceinline__ DF df_fma(DF a, DF b, DF acc) { return df_add(acc, df_mul(a, b)); }

// ---- packed FP32 pairs (sm_100+) -----------------------------------------
// c + a * b on both halves of a float2 in one instruction (CUDA's
// __ffma2_rn); each half is the IEEE fma of that half, so results equal two
// scalar fmaf calls.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// ---- asynchronous global -> shared copies (sm_80+) ------------------------
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// ---- tensor memory access (TMA) and mbarriers (sm_90+) --------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// Waits for phase `parity` of the barrier; gives up after `tries` polls
// (each poll may itself wait a short, hardware-chosen time) and returns false.
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity, int tries) {
  for (int i = 0; i < tries; ++i) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
// One tiled TMA load of a box at (c0, c1[, c2[, c3]]) of the tensor
// described by `map` (a __grid_constant__ CUtensorMap) into shared memory,
// completing on `bar`.
__device__ __forceinline__ void tma_load2(void* dst, const void* map, int c0, int c1,
                                          unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load3(void* dst, const void* map, int c0, int c1, int c2,
                                          unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
      "%4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load4(void* dst, const void* map, int c0, int c1, int c2, int c3,
                                          unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
      "%4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// ---- atomics ---------------------------------------------------------------
// Complex add into global memory: one vector reduction for FP32 (sm_90+),
// two scalar reductions for FP64.
__device__ __forceinline__ void red_add(float2* p, float re, float im) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(re), "f"(im) : "memory");
}
__device__ __forceinline__ void red_add(double2* p, double re, double im) {
  atomicAdd(&p->x, re);
  atomicAdd(&p->y, im);
}

// Shared-memory complex add.
__device__ __forceinline__ void smem_add(float2* p, float re, float im) {
  atomicAdd(&p->x, re);
  atomicAdd(&p->y, im);
}
__device__ __forceinline__ void smem_add(double2* p, double re, double im) {
  atomicAdd(&p->x, re);
  atomicAdd(&p->y, im);
}

__device__ __forceinline__ int wrap_idx(int i, int n) {
  if (i >= n) i -= n;
  return i;
}

}  // namespace cfg
