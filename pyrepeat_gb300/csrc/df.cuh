// Double-float arithmetic on the FP32 pipe.
//
// A value is carried as an unevaluated sum hi + lo of two floats.  Products and
// sums use the classical error-free transformations: TwoSum (Knuth, TAOCP vol. 2,
// 4.2.2), Fast2Sum (Dekker 1971) and the FMA form of TwoProd (the rounding error
// of a*b is fma(a, b, -a*b) exactly).  The explicit __fadd_rn / __fmul_rn
// intrinsics keep the compiler from contracting the rounded product or sum
// into an FMA, which would break the transformations.
//
// An accumulator keeps the running FP32 sum `s` and, in `e`, every rounding
// error of the additions plus the low-order part of every product, so a sum of
// n terms is exact to about 2^-46 of the largest partial sum: far below what the
// fit needs, at roughly ten FP32 operations per multiply-add (FP64 runs at a small
// fraction of the FP32 rate on this part).
#pragma once

namespace rp {
namespace dfa {

struct acc {
    float s, e;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &err) {
    s = __fadd_rn(a, b);
    const float bb = __fadd_rn(s, -a);
    err = __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb));
}

// c += (ah + al) * (bh + bl), dropping only al * bl (2^-48 relative)
__device__ __forceinline__ void mac(acc &c, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    float pe = __fmaf_rn(ah, bh, -p);
    pe = __fmaf_rn(ah, bl, pe);
    pe = __fmaf_rn(al, bh, pe);
    float s, err;
    two_sum(c.s, p, s, err);
    c.s = s;
    c.e = __fadd_rn(c.e, __fadd_rn(err, pe));
}

// the accumulated value as a normalised pair (hi, lo) with |lo| <= ulp(hi)/2
__device__ __forceinline__ float2 norm(const acc &c) {
    const float h = __fadd_rn(c.s, c.e);
    const float l = __fadd_rn(c.e, -__fadd_rn(h, -c.s));
    return make_float2(h, l);
}

__device__ __forceinline__ double to_double(const acc &c) { return (double)c.s + (double)c.e; }

// complex multiply-accumulate: (re, im) += x * y with x = (xr, xi), y = (yr, yi), each part a
// double-float stored as float4 (re_h, re_l, im_h, im_l)
__device__ __forceinline__ void cmac(acc &re, acc &im, const float4 &x, const float4 &y) {
    mac(re, x.x, x.y, y.x, y.y);
    mac(re, -x.z, -x.w, y.z, y.w);
    mac(im, x.x, x.y, y.z, y.w);
    mac(im, x.z, x.w, y.x, y.y);
}

// real part only: re += Re(x * y)
__device__ __forceinline__ void cmac_re(acc &re, const float4 &x, const float4 &y) {
    mac(re, x.x, x.y, y.x, y.y);
    mac(re, -x.z, -x.w, y.z, y.w);
}

// FP32 forms (hi parts only): stage B of the separable sum and the per-point stage C use
// these; their rounding errors are unbiased and ~1e-7 relative, the level of the FP32
// real-space terms, and measured to leave the fitted charges unchanged at 1e-7 e.
__device__ __forceinline__ void cmac32(float &re, float &im, const float4 &x, const float4 &y) {
    re = fmaf(x.x, y.x, re);
    re = fmaf(-x.z, y.z, re);
    im = fmaf(x.x, y.z, im);
    im = fmaf(x.z, y.x, im);
}

__device__ __forceinline__ float cre32(float re, const float4 &x, const float4 &y) {
    re = fmaf(x.x, y.x, re);
    return fmaf(-x.z, y.z, re);
}

__device__ __forceinline__ float4 pack(const acc &re, const acc &im) {
    const float2 r = norm(re), i = norm(im);
    return make_float4(r.x, r.y, i.x, i.y);
}

// FP64 complex value -> double-float float4
__host__ __device__ inline float4 split(double re, double im) {
    const float rh = (float)re, ih = (float)im;
    return make_float4(rh, (float)(re - (double)rh), ih, (float)(im - (double)ih));
}

}  // namespace dfa
}  // namespace rp
