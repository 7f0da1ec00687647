// mixed_ops.cuh -- operand splitting, swizzled tile layout and compensated sums shared by the
// tensor-core kernels (vxc_mixed.cu, xc_grad_mixed.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "dfloat.cuh"
#include "tc_ptx.cuh"

namespace cxc {
namespace mix {

constexpr int kThreads = 256;  // threads per CTA of the tensor-core kernels
constexpr int kNc = 64;        // GEMM1 N chunk (AOs) per TMEM accumulator

__device__ __forceinline__ uint32_t pack_bf16x2(__nv_bfloat16 a, __nv_bfloat16 b) {
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// x = hi + mid + lo, each an RN BF16 of the remaining residual; the residuals are exact in FP32.
__device__ __forceinline__ void split3_bf16(float x, __nv_bfloat16& hi, __nv_bfloat16& mid, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(hi);
  mid = __float2bfloat16_rn(r1);
  lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
}

__device__ __forceinline__ uint32_t bf162_bits(__nv_bfloat162 v) {
  return (uint32_t)__bfloat16_as_ushort(v.x) | ((uint32_t)__bfloat16_as_ushort(v.y) << 16);
}

// split3_bf16 of eight values, two at a time (one paired conversion per piece): the same pieces,
// packed in order (value 2k in the low half of word k)
__device__ __forceinline__ void pack8x3(const float* v, uint4& hi, uint4& mid, uint4& lo) {
  uint32_t h[4], md[4], l[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float a = v[2 * k], b = v[2 * k + 1];
    const __nv_bfloat162 h2 = __floats2bfloat162_rn(a, b);
    const float ra = __fsub_rn(a, __low2float(h2)), rb = __fsub_rn(b, __high2float(h2));
    const __nv_bfloat162 m2 = __floats2bfloat162_rn(ra, rb);
    const __nv_bfloat162 l2 = __floats2bfloat162_rn(__fsub_rn(ra, __low2float(m2)), __fsub_rn(rb, __high2float(m2)));
    h[k] = bf162_bits(h2);
    md[k] = bf162_bits(m2);
    l[k] = bf162_bits(l2);
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  mid = make_uint4(md[0], md[1], md[2], md[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// Fixed-point split of |x| < 1 (a double-float hi + lo) into four pieces that are multiples of
// 2^-7, 2^-15, 2^-23 and 2^-31 with at most 8 significant bits each (exact in BF16); the residual
// x - (h + m + l + q) is below 2^-32.
__device__ __forceinline__ void fixsplit4(float xh, float xl, __nv_bfloat16& hi, __nv_bfloat16& mid,
                                          __nv_bfloat16& lo, __nv_bfloat16& q) {
  const float h = rintf(xh * 128.f) * (1.f / 128.f);
  const float r1 = __fadd_rn(__fsub_rn(xh, h), xl);
  const float m = rintf(r1 * 32768.f) * (1.f / 32768.f);
  const float r2 = __fsub_rn(r1, m);
  const float l = rintf(r2 * 8388608.f) * (1.f / 8388608.f);
  const float r3 = __fsub_rn(r2, l);
  const float qq = rintf(r3 * 2147483648.f) * (1.f / 2147483648.f);
  hi = __float2bfloat16_rn(h);
  mid = __float2bfloat16_rn(m);
  lo = __float2bfloat16_rn(l);
  q = __float2bfloat16_rn(qq);
}

__device__ __forceinline__ uint4 pack8v(const __nv_bfloat16* v) {
  return make_uint4(pack_bf16x2(v[0], v[1]), pack_bf16x2(v[2], v[3]), pack_bf16x2(v[4], v[5]), pack_bf16x2(v[6], v[7]));
}

// Byte offset of 16-byte chunk c (0..7) of row r in a 128-byte-swizzled K-major tile.
__device__ __forceinline__ uint32_t sw128(int r, int c) { return (uint32_t)(r * 128 + ((c ^ (r & 7)) << 4)); }

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint4 v) {
  asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}

// GEMM1 B operand for K block kb and N chunk [nc, nc + N): D[nu][mu] 2^-f_nu pieces hi / mid / lo
// / lo2 at stage + 64 KB + q * N * 128 (N rows x 64 K, 128-byte swizzle), gathered from the packed
// fixed-point density (x = hi | mid << 16, y = lo | lo2 << 16).
template <int N = kNc>
static __device__ void gather_b(unsigned char* stage, const uint2* __restrict__ Dp, const int* s_ao, int n, int m, int kb,
                         int nc) {
  constexpr uint32_t kPiece = N * 128;
  const uint32_t sbase = smem_addr(stage) + 65536;
  for (int e = threadIdx.x; e < N * 8; e += kThreads) {
    const int c = e & 7, r = e >> 3;
    const int nu = nc + r;
    const int mu0 = kb * 64 + c * 8;
    uint32_t hw[4] = {0, 0, 0, 0}, mw[4] = {0, 0, 0, 0}, lw[4] = {0, 0, 0, 0}, qw[4] = {0, 0, 0, 0};
    if (nu < m) {
      const uint2* row = Dp + (size_t)s_ao[nu] * n;
#pragma unroll
      for (int k = 0; k < 8; k += 2) {
        const uint2 a = (mu0 + k < m) ? __ldg(row + s_ao[mu0 + k]) : make_uint2(0u, 0u);
        const uint2 b = (mu0 + k + 1 < m) ? __ldg(row + s_ao[mu0 + k + 1]) : make_uint2(0u, 0u);
        hw[k >> 1] = (a.x & 0xFFFFu) | (b.x << 16);
        mw[k >> 1] = (a.x >> 16) | (b.x & 0xFFFF0000u);
        lw[k >> 1] = (a.y & 0xFFFFu) | (b.y << 16);
        qw[k >> 1] = (a.y >> 16) | (b.y & 0xFFFF0000u);
      }
    }
    const uint32_t off = sw128(r, c);
    st_shared_v4(sbase + off, make_uint4(hw[0], hw[1], hw[2], hw[3]));
    st_shared_v4(sbase + kPiece + off, make_uint4(mw[0], mw[1], mw[2], mw[3]));
    st_shared_v4(sbase + 2 * kPiece + off, make_uint4(lw[0], lw[1], lw[2], lw[3]));
    st_shared_v4(sbase + 3 * kPiece + off, make_uint4(qw[0], qw[1], qw[2], qw[3]));
  }
}

// Compensated sum of double-float products: s collects the FP32 parts by TwoSum, c every rounding
// and low-order term (Ogita-Rump-Oishi Sum2 applied to the TwoProd pieces).
struct CompSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

__device__ __forceinline__ void acc_prod(CompSum& A, df32 x, df32 t) {
  const float p = __fmul_rn(x.hi, t.hi);
  float e = __fmaf_rn(x.hi, t.hi, -p);
  e = __fmaf_rn(x.hi, t.lo, __fmaf_rn(x.lo, t.hi, e));
  const df32 q = two_sum(A.s, p);
  A.s = q.hi;
  A.c = __fadd_rn(A.c, __fadd_rn(q.lo, e));
}

// The same product summed by FP32 FMAs: s collects x.hi t.hi, c the cross terms x.hi t.lo +
// x.lo t.hi; the rounding of each FMA into s is not recovered.  The double-float value's low part
// still enters (its error is the same at every point of a radial shell and would not average out);
// the accumulation's own roundings vary from point to point.
__device__ __forceinline__ void acc_prod_fma(CompSum& A, df32 x, df32 t) {
  A.s = __fmaf_rn(x.hi, t.hi, A.s);
  A.c = __fmaf_rn(x.hi, t.lo, __fmaf_rn(x.lo, t.hi, A.c));
}

}  // namespace mix
}  // namespace cxc
