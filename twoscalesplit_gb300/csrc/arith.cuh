// arith.cuh -- the two arithmetic policies of the gathers' per-pair work.
//
// ExactArith is the reference's arithmetic: every expression in the reference's
// FP32 association, IEEE square root and division, no contraction (the functions
// of tss_device.cuh), so a gather gives the reference's bits for the same
// summation order.  It is the default and the parity path.
//
// FastArith spends the tolerance the step is specified to (1e-5 relative in FP32
// for densities, forces and positions) instead of bit-exactness.  Per pair it takes
// one approximate reciprocal square root (d = x * rsqrt(x)), one approximate
// reciprocal (the viscosity denominator) and fused multiply-adds; the cubic spline
// and its gradient are written in expanded form, which removes the IEEE divisions
// of the gradient (n / d): for q < 1 the gradient's numerator has the factor q =
// 2d/r, so n/d = G (2/r) (4 - 3q); for 1 <= q < 2 it is G (2 - q)^2 / d = G (2 -
// q)^2 rsqrt(x).  Summation order, cutoffs (tested on the squared distance, as in
// the exact path), neighbour sets and all integer grid work are the same as in the
// exact path; only the value of each pair's term differs, by a few units in the
// last place.  The per-particle quantities (Tait pressure, p/rho^2, integration,
// split test, tether) stay in the exact arithmetic.
//
// Algebra (2D cubic spline, support radius r, q = 2d/r, WCSPHSolver.cu:116-239):
//   (2-q)^3 - 4(1-q)^3 = 4 - 6q^2 + 3q^3 = 4 + q^2 (3q - 6)
//   (2-q)^2 - 4(1-q)^2 = 4q - 3q^2      = q (4 - 3q)
// The approximate operations are the PTX instructions rsqrt.approx.ftz.f32,
// sqrt.approx.ftz.f32 and rcp.approx.ftz.f32 (PTX ISA: relative error of a few
// 2^-23); their arguments here are squared distances and sums of positive
// densities, never subnormal except for pairs closer than ~1e-19, which the force
// sums exclude by their x != 0 test and the density takes as d = 0.
#pragma once
#include "tss_device.cuh"

namespace tss {

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sqrt_approx(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Viscosity lengths of the force sums: 0 = r (low-low), 1 = (r + rh)/2 (cross
// scale), 2 = rh (high-high).
enum { kHLow = 0, kHCross = 1, kHHigh = 2 };

struct ExactArith {
    static constexpr bool kFast = false;

    template <int HS>
    __device__ __forceinline__ static PairTerms pair(const Params& P, float2 pij, float x, float2 vij, float qi,
                                                     float qj, float densi, float densj) {
        const float h = HS == kHLow ? P.r : (HS == kHCross ? P.hx : P.rh);
        return pair_terms(P, pij, sqrtf(x), vij, qi, qj, densi, densj, h);
    }

    __device__ __forceinline__ static float density(const Params& P, float x) { return pair_density(P, sqrtf(x)); }

    // wall term of scale S (0: r, 1: rh): cB * Gamma_rad(d) * pik
    template <int S>
    __device__ __forceinline__ static float2 wall(const Params& P, float2 pik, float x, float cB) {
        const float rad = S ? P.rh : P.r;
        const float yh = S ? P.inv_hi.y : P.inv_hi.x, yl = S ? P.inv_lo.y : P.inv_lo.x;
        const float d = sqrtf(x);
        const float gm = wall_weight_q(d, div_const(d * 2.0f, rad, yh, yl), P.cs);
        return make_float2(cB * gm * pik.x, cB * gm * pik.y);
    }
};

// Every value FastArith hands to a sum (the pair's terms, a kernel's two halves)
// comes from the scalar __fmul_rn / __fadd_rn intrinsics, which are never merged
// into a fused multiply-add, so the bits do not depend on how the compiler
// schedules one kernel form or another: the batched and single-scene forms, and
// the one-particle-per-thread and per-warp walks, give the same results, as in the
// exact arithmetic.  (--fmad=false does not keep a packed product apart from the
// packed add it feeds: that was measured in the exact arithmetic's kernel pairs.)
struct FastArith {
    static constexpr bool kFast = true;

    // Both scales' kernel and gradient factors at q = (2d/r, 2d/rh), already scaled
    // by the halved coefficients (P.fC = C/2, P.fG = G/2): w = W_r/2 + W_rh/2 and
    // c = (dW_r/dd + dW_rh/dd) / (2d), so that a pair's gradient term is c * x_ij.
    __device__ __forceinline__ static void kernels(const Params& P, float x, float rinv, float d, float& w,
                                                   float& c) {
        const float2 tor = P.fTor;
        const float2 q = __fmul2_rn(make_float2(d, d), tor);
        const float2 q2 = __fmul2_rn(q, q);
        const float2 t = __ffma2_rn(q, make_float2(3.0f, 3.0f), make_float2(-6.0f, -6.0f));
        const float2 w1 = __ffma2_rn(q2, t, make_float2(4.0f, 4.0f));
        const float2 g1 = __fmul2_rn(__ffma2_rn(q, make_float2(-3.0f, -3.0f), make_float2(4.0f, 4.0f)), tor);
        const float2 a = __ffma2_rn(q, make_float2(-1.0f, -1.0f), make_float2(2.0f, 2.0f));
        const float2 aa = __fmul2_rn(a, a);
        const float2 w2 = __fmul2_rn(aa, a);
        const float2 g2 = __fmul2_rn(aa, make_float2(rinv, rinv));
        const float2 ws = make_float2(q.x < 1.0f ? w1.x : (q.x < 2.0f ? w2.x : 0.0f),
                                      q.y < 1.0f ? w1.y : (q.y < 2.0f ? w2.y : 0.0f));
        const float2 gs = make_float2(q.x < 1.0f ? g1.x : (q.x < 2.0f ? g2.x : 0.0f),
                                      q.y < 1.0f ? g1.y : (q.y < 2.0f ? g2.y : 0.0f));
        w = __fadd_rn(__fmul_rn(ws.x, P.fC.x), __fmul_rn(ws.y, P.fC.y));
        c = __fadd_rn(__fmul_rn(gs.x, P.fG.x), __fmul_rn(gs.y, P.fG.y));
    }

    template <int HS>
    __device__ __forceinline__ static PairTerms pair(const Params& P, float2 pij, float x, float2 vij, float qi,
                                                     float qj, float densi, float densj) {
        const float rinv = rsqrt_approx(x);
        const float d = __fmul_rn(x, rinv);
        float w, c;
        kernels(P, x, rinv, d, w, c);
        const float dvp = __fmaf_rn(vij.x, pij.x, __fmul_rn(vij.y, pij.y));
        const float eps = HS == kHLow ? P.fEps.x : (HS == kHCross ? P.fEps.y : P.fEps.z);
        const float kv = HS == kHLow ? P.fKv.x : (HS == kHCross ? P.fKv.y : P.fKv.z);
        const float den = __fmul_rn(__fadd_rn(x, eps), __fadd_rn(densi, densj));
        const float visc = __fmul_rn(__fmul_rn(dvp, kv), rcp_approx(den));
        const float qs = __fadd_rn(qi, qj);
        const float coeff = dvp < 0.0f ? __fsub_rn(qs, visc) : qs;
        const float s = __fmul_rn(coeff, c);
        return PairTerms{make_float2(__fmul_rn(s, pij.x), __fmul_rn(s, pij.y)),
                         make_float2(__fmul_rn(w, pij.x), __fmul_rn(w, pij.y))};
    }

    // (W_r(d) + W_rh(d)) / 2 at d = sqrt(x)
    __device__ __forceinline__ static float density(const Params& P, float x) {
        const float d = sqrt_approx(x);
        const float2 q = __fmul2_rn(make_float2(d, d), P.fTor);
        const float2 q2 = __fmul2_rn(q, q);
        const float2 t = __ffma2_rn(q, make_float2(3.0f, 3.0f), make_float2(-6.0f, -6.0f));
        const float2 w1 = __ffma2_rn(q2, t, make_float2(4.0f, 4.0f));
        const float2 a = __ffma2_rn(q, make_float2(-1.0f, -1.0f), make_float2(2.0f, 2.0f));
        const float2 w2 = __fmul2_rn(__fmul2_rn(a, a), a);
        const float2 ws = make_float2(q.x < 1.0f ? w1.x : (q.x < 2.0f ? w2.x : 0.0f),
                                      q.y < 1.0f ? w1.y : (q.y < 2.0f ? w2.y : 0.0f));
        return __fadd_rn(__fmul_rn(ws.x, P.fC.x), __fmul_rn(ws.y, P.fC.y));
    }

    // Gamma_rad(d) = 0.02 c^2 / d^2 * {2/3; 2q - 1.5q^2 = q (2 - 1.5q); 0.5 (2-q)^2; 0}
    template <int S>
    __device__ __forceinline__ static float2 wall(const Params& P, float2 pik, float x, float cB) {
        const float d = sqrt_approx(x);
        const float q = __fmul_rn(d, S ? P.fTor.y : P.fTor.x);
        const float a = __fsub_rn(2.0f, q);
        const float r2 = __fmul_rn(q, __fmaf_rn(-1.5f, q, 2.0f));
        const float r3 = __fmul_rn(__fmul_rn(0.5f, a), a);
        const float f = q < 2.0f / 3.0f ? 2.0f / 3.0f : (q < 1.0f ? r2 : (q < 2.0f ? r3 : 0.0f));
        const float gm = __fmul_rn(__fmul_rn(__fmul_rn(cB, P.fKw), rcp_approx(x)), f);
        return make_float2(__fmul_rn(gm, pik.x), __fmul_rn(gm, pik.y));
    }
};

}  // namespace tss
