// Sums of products in FP32 with FP64-class accuracy ("double-float").
//
// The dense coarsest-level solve of the FP32 V-cycle is x = T r with T the
// inverse of an ill-conditioned coarse matrix (condition ~1e5-1e7 on 3D
// hierarchies): its rows hold large entries of both signs whose products
// cancel, so a plain FP32 sum loses the correction (relative error ~1e-3 on
// a 64^3 P1 hierarchy, enough to stall the outer CG).  FP64 arithmetic would
// fix it but runs at a small fraction of the FP32 rate on this GPU.  Instead
// T is stored as an unevaluated pair T = hi + lo of FP32 arrays (same bytes
// as FP64) and each row is accumulated as a pair (sh, sl):
//   - the product hi*v is split exactly into p + e with one FMA (TwoProd),
//   - p is added to sh with Knuth's TwoSum, whose rounding error is exact,
//   - the small parts (TwoSum error, e, lo*v) are summed into sl in FP32.
// The __f*_rn intrinsics keep the compiler from contracting the exact steps
// into FMAs, which would break the error-free transforms.
#pragma once

namespace afp {

// s + e == a + b exactly (Knuth's TwoSum, no ordering requirement)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float z = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z));
}

// (sh, sl) += (hi + lo) * v
__device__ __forceinline__ void df_add_prod(float& sh, float& sl, float hi, float lo, float v) {
  const float p = __fmul_rn(hi, v);
  const float pe = __fmaf_rn(hi, v, -p);  // hi*v - p, exact
  float s, e;
  two_sum(sh, p, s, e);
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(e, __fmaf_rn(lo, v, pe)));
}

// (sh, sl) += (oh, ol)
__device__ __forceinline__ void df_add(float& sh, float& sl, float oh, float ol) {
  float s, e;
  two_sum(sh, oh, s, e);
  sh = s;
  sl = __fadd_rn(sl, __fadd_rn(ol, e));
}

}  // namespace afp
