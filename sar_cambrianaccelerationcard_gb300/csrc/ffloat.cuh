// ffloat.cuh -- float-float ("double-float") arithmetic on the FP32 pipe:
// a value is h + l with |l| <= ulp(h)/2, about 48 significant bits.
// Error-free transforms: Knuth two-sum and the FMA two-product.  Used where
// FP64 would run on GB300's narrow FP64 pipe: back-projection's per-(tile,
// pulse) references (bp.cu) and the omega-K phase (wk.cu).
#pragma once

namespace sarbp {
namespace {

struct ff {
    float h, l;
};
__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ ff quick_two_sum(float a, float b) {
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const ff s = two_sum(a.h, b.h);
    return quick_two_sum(s.h, s.l + (a.l + b.l));
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const float p = a.h * b;
    const float e = fmaf(a.h, b, -p);
    return quick_two_sum(p, fmaf(a.l, b, e));
}

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = a.h * b.h;
    const float e = fmaf(a.h, b.h, -p);
    return quick_two_sum(p, e + fmaf(a.h, b.l, a.l * b.h));
}

// v modulo 2 pi, in [-pi, pi], rounded to float (2 pi as a float pair).
__device__ __forceinline__ float ff_mod_2pi(ff v) {
    const ff twopi = {6.28318548202514648f, -1.7484555314695172e-07f};
    const float n = rintf(v.h * 0.159154943091895336f);
    const ff r = ff_add(v, ff_mul_f(twopi, -n));
    return r.h + r.l;
}

}  // namespace
}  // namespace sarbp
