// tss_device.cuh -- device-side types and per-pair arithmetic of the two-scale
// WCSPH step.  Every expression keeps the reference's FP32 operation order
// (TwoScale2D/WCSPHSolver.cu:66-333, 476-954) and the library is compiled with
// --fmad=false and IEEE division/square root, so a kernel's result is the
// reference's result for the same summation order, bit for bit.
#pragma once
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace tss {

constexpr double kPi = 3.14159265358979323846;  // WCSPHSolver.cu:19

// error word bits (mirror TSS_ERR_* in include/tss.h)
constexpr unsigned kErrCapacity = 0x1u;
constexpr unsigned kErrNumeric = 0x2u;
constexpr unsigned kErrGridIndex = 0x4u;  // a grid index check failed: inconsistent cell offsets

struct Params {
    float ox, oy;
    int dimL[2], dimH[2];
    float r, rh, rho0, B, cs, alpha, sigma, dt, g;
    float CL, GL, CH, GH;  // kernel / gradient coefficients (Bind, WCSPHSolver.cu:2559-2590)
    float mL, mH, mB;
    float cBL, cBH;        // mB/(mL+mB), mB/(mH+mB)
    float hx;              // (r + rh) / 2, the cross-scale viscosity length
    float relax_dt;
    float roi[4];
    float roi_vdt[2];      // ROI displacement per step (roi_velocity * dt)
    int relax_iters;
    int q1;
    int merge;             // TSS_FLAG_MERGE
    int tether_guard;      // TSS_FLAG_TETHER_GUARD
    int older_place;       // TSS_FLAG_OLDER_PLACEMENT
    long long step0;       // the step counter when the scene started (its ROI's step 0)
    int slotsL, slotsH;    // slot-id spaces: low ids < slotsL, high ids < slotsH = 4*slotsL
    int capH;
    // scene placement in a batch (all zero for a single scene): cell bases of the
    // scene's low/high grids in the global cell space, its first low-res slot id,
    // its low-res particle count, high-res cell count and first wall particle (the
    // scene's wall cell offsets count from it)
    int cbL, cbH, sbL, nLs, CHs, wb;
    // exact squared-distance cutoffs: x <= Tle_s  <=>  sqrtf(x) <= r_s and
    // x <= Tlt_s  <=>  sqrtf(x) < r_s, for x = dx*dx + dy*dy (IEEE sqrt is monotone
    // and correctly rounded, so these are the largest floats with that property)
    float Tle_r, Tlt_r, Tle_rh, Tlt_rh;
    // reciprocal splits of (r, rh) for div_const: hi = RN(1/r_s), lo = RN(1/r_s - hi)
    float2 inv_hi, inv_lo;
    // constants of the tolerance arithmetic (FastArith, arith.cuh): (2/r, 2/rh),
    // the halved kernel and gradient coefficients (C/2, G/2) of both scales, the
    // viscosity's 0.01 h^2 and 2 h alpha c for h = r, (r + rh)/2, rh, and the wall
    // weight's 0.02 c^2
    float2 fTor, fC, fG;
    float3 fEps, fKv;
    float fKw;
};

// Division by a per-scene constant b (the smoothing lengths), correctly rounded:
// the IEEE quotient RN(a/b) from the reciprocal split yh = RN(1/b), yl ~ 1/b - yh
// (recip_split), in three fused multiply-adds and a multiply:
//   q0 = RN(a*yh + RN(a*yl))   a*(yh + yl) is a/b to ~2^-47, so q0 is within one ulp
//   r  = a - q0*b              exact: the remainder of a quotient within one ulp
//   q  = RN(q0 + r*yh)         = RN(a/b) by Markstein's theorem (yh within half an
//                              ulp of 1/b, q0 within one ulp of a/b)
// (P. W. Markstein, "Computation of elementary functions on the IBM RISC
// System/6000 processor", IBM J. Res. Develop. 34(1):111-119, 1990; J.-M. Muller
// et al., Handbook of Floating-Point Arithmetic, chapter on division with an FMA.)
// The theorem needs every step in the normal range.  The callers divide a = 2d by
// r and by rh, d the distance of a pair in range (0 <= d <= r, so a <= 4b; the
// square root of a float, so +0 or >= 2^-75), with r and rh in [2^-40, 2^40] (the
// configuration check); a NaN a gives NaN, as the division does.  One input
// differs: a = -0 gives +0 when yl < 0 (a*yl is then +0), where the division gives
// -0; the callers never divide -0.  tests/cuda/div_const.cu
// compares both forms with the IEEE division on every float |a| <= 16b for a set of
// divisors, bit for bit.
__device__ __forceinline__ float div_const(float a, float b, float yh, float yl) {
    const float q0 = __fmaf_rn(a, yh, __fmul_rn(a, yl));
    const float r = __fmaf_rn(-q0, b, a);
    return __fmaf_rn(r, yh, q0);
}

// both scales at once: (a.x / b.x, a.y / b.y), as f32x2 pairs
__device__ __forceinline__ float2 div_const2(float2 a, float2 b, float2 yh, float2 yl) {
    const float2 q0 = __ffma2_rn(a, yh, __fmul2_rn(a, yl));
    const float2 r = __ffma2_rn(make_float2(-q0.x, -q0.y), b, a);
    return __ffma2_rn(r, yh, q0);
}

// The reciprocal split of b > 0 for div_const (host).  For floats b and y the
// product b*y has at most 48 significant bits, so 1 - b*y is exact in double and
// |1 - b*y| = b*|1/b - y| ranks the three floats around the double reciprocal by
// their distance to 1/b exactly: yh is the nearest, RN(1/b).
inline void recip_split(float b, float& yh, float& yl) {
    const double bd = b;
    const float y0 = static_cast<float>(1.0 / bd);
    const float cand[3] = {y0, std::nextafterf(y0, 0.0f), std::nextafterf(y0, INFINITY)};
    yh = y0;
    double best = std::fabs(1.0 - bd * static_cast<double>(y0));
    for (float c : cand) {
        const double e = std::fabs(1.0 - bd * static_cast<double>(c));
        if (e < best) {
            best = e;
            yh = c;
        }
    }
    yl = static_cast<float>((1.0 - bd * static_cast<double>(yh)) / bd);
}

// Device-side counters of one solver.  `cur` is what this step's kernels use;
// `next` is what the step produces; the step's last kernel copies next -> cur.
struct Counters {
    int cur[2];
    int next[2];
    int n_fresh;     // parents split in the previous step (relaxed this step)
    int n_split;     // parents split in this step
    unsigned err;    // kErr* bits
    int h_state0;    // 1 if some high-res particle has (state & 1) == 0
    long long steps;
    int sorted[2];   // particles sorted in the last step (its `cur` counts)
    int n_drop;      // high-res list entries removed (state 2) in this step
    int dropped;     // ... in the last step: they are still in the list until the next build
    long long total_split;    // splits since creation
    long long total_removed;  // high-res particles removed by merges since creation
};

__device__ __forceinline__ int f2i(float v) { return static_cast<int>(v); }  // cvt.rzi: trunc, saturating

// Packed FP32 pairs: sm_100's two-wide add and multiply (__fadd2_rn, __fmul2_rn)
// round each component exactly as the scalar operation.  --fmad=false keeps the
// scalar multiplies and adds apart, but not the packed ones: a packed product used
// once and fed to a packed add or subtract was measured to come out as one packed
// fused multiply-add.  So no packed product here feeds a packed add or subtract
// directly, except an exact product (by 0.5, where fusing changes nothing); such
// a difference is taken in scalar, and the parity tests pin every result to the
// scalar expression bit for bit.  a - b is a + (-b) (IEEE defines subtraction so).
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }

// computeGridCoordinate(pos, offset), WCSPHSolver.cu:265-289
__device__ __forceinline__ void grid_coord(float px, float py, float off, float ox, float oy, float cell,
                                           int dimx, int dimy, int& cx, int& cy) {
    cx = f2i(((px + off) - ox) / cell);
    cy = f2i(((py + off) - oy) / cell);
    cx = min(max(0, cx), dimx - 1);
    cy = min(max(0, cy), dimy - 1);
}

__device__ __forceinline__ int cell_hash(float2 p, float ox, float oy, float cell, int dimx, int dimy) {
    int cx, cy;
    grid_coord(p.x, p.y, 0.0f, ox, oy, cell, dimx, dimy, cx, cy);
    return cy * dimx + cx;
}

// computeGridCoordinate on grid S of a scene (0: the low-res grid, cell r; 1: the
// high-res grid, cell rh), the quotient by the cell size taken with div_const.  A
// cell index needs only the truncation of the IEEE quotient, and div_const gives
// that for every finite a: it is the IEEE quotient for 2^-75 <= |a| (the quotient
// then normal), and for smaller |a| both quotients are below 2^-35 and truncate
// to 0.  An infinite or NaN a keeps the division's result, a itself (the cell size
// is positive and finite).
__device__ __forceinline__ float cell_quot(float a, float cell, float yh, float yl) {
    return isfinite(a) ? div_const(a, cell, yh, yl) : a;
}

template <int S>
__device__ __forceinline__ void grid_coord_s(const Params& P, float px, float py, float off, int& cx, int& cy) {
    const float cell = S ? P.rh : P.r;
    const float yh = S ? P.inv_hi.y : P.inv_hi.x, yl = S ? P.inv_lo.y : P.inv_lo.x;
    const int dimx = S ? P.dimH[0] : P.dimL[0], dimy = S ? P.dimH[1] : P.dimL[1];
    cx = f2i(cell_quot((px + off) - P.ox, cell, yh, yl));
    cy = f2i(cell_quot((py + off) - P.oy, cell, yh, yl));
    cx = min(max(0, cx), dimx - 1);
    cy = min(max(0, cy), dimy - 1);
}

template <int S>
__device__ __forceinline__ int cell_hash_s(const Params& P, float2 p) {
    int cx, cy;
    grid_coord_s<S>(P, p.x, p.y, 0.0f, cx, cy);
    return cy * (S ? P.dimH[0] : P.dimL[0]) + cx;
}

// evaluateM4Kernel(High), WCSPHSolver.cu:116-160.  Both polynomial branches are
// evaluated and one is selected: each branch's expression keeps the reference's
// association, so the selected value is the reference's bit for bit, and a warp
// whose lanes fall into different branches does not run both in turn.
__device__ __forceinline__ float kernW(float d, float rad, float C) {
    const float q = d * 2.0f / rad;
    const float a = 2.0f - q, b = 1.0f - q;
    const float w1 = C * (a * a * a - 4.0f * b * b * b);
    const float w2 = C * a * a * a;
    return q < 1.0f ? w1 : (q < 2.0f ? w2 : 0.0f);
}

// evaluateGradientM4Kernel(High), WCSPHSolver.cu:162-239: c = G*(a*a - 4*b*b)/d for
// q < 1 and c = G*a*a/d for q < 2 -- one division of the selected numerator.
__device__ __forceinline__ float2 kernDW(float2 x, float d, float rad, float G) {
    const float q = d * 2.0f / rad;
    const float a = 2.0f - q, b = 1.0f - q;
    const float n1 = G * (a * a - 4.0f * b * b);
    const float n2 = G * a * a;
    const float c = (q < 1.0f ? n1 : n2) / d;
    return q < 2.0f ? mul2(make_float2(c, c), x) : make_float2(0.0f, 0.0f);
}

// Both scales' kernels at one distance d, packed in pairs: x is the low-res scale
// (r, CL, GL), y the high-res scale (rh, CH, GH).  Each half is the scalar
// expression of kernW / kernDW above -- the same operations in the same
// association ((a*a)*a, ((4*b)*b)*b, ((C*a)*a)*a, (G*a)*a), each rounded once --
// so each half equals the scalar value bit for bit.
struct Kern2 {
    float2 q, a, b, aa, fbb;  // q = 2d/rad, a = 2 - q, b = 1 - q, a*a, (4*b)*b
};

__device__ __forceinline__ Kern2 kern2(float d, const Params& P) {
    Kern2 k;
    const float d2 = d * 2.0f;
    k.q = div_const2(make_float2(d2, d2), make_float2(P.r, P.rh), P.inv_hi, P.inv_lo);  // (d2 / r, d2 / rh)
    k.a = sub2(make_float2(2.0f, 2.0f), k.q);
    k.b = sub2(make_float2(1.0f, 1.0f), k.q);
    k.aa = mul2(k.a, k.a);
    k.fbb = mul2(mul2(make_float2(4.0f, 4.0f), k.b), k.b);
    return k;
}

// evaluateM4Kernel of both scales: C * (a*a*a - 4*b*b*b) for q < 1, C*a*a*a for q < 2
// (the difference of the two products in scalar: see add2 above)
__device__ __forceinline__ float2 kernW2(const Kern2& k, float2 C) {
    const float2 a3 = mul2(k.aa, k.a), b3 = mul2(k.fbb, k.b);
    const float2 w1 = mul2(C, make_float2(a3.x - b3.x, a3.y - b3.y));
    const float2 w2 = mul2(mul2(mul2(C, k.a), k.a), k.a);
    return make_float2(k.q.x < 1.0f ? w1.x : (k.q.x < 2.0f ? w2.x : 0.0f),
                       k.q.y < 1.0f ? w1.y : (k.q.y < 2.0f ? w2.y : 0.0f));
}

// evaluateGradientM4Kernel of both scales applied to x: gI (low-res), gJ (high-res)
__device__ __forceinline__ void kernDW2(const Kern2& k, float2 G, float2 x, float d, float2& gI, float2& gJ) {
    const float2 n1 = mul2(G, make_float2(k.aa.x - k.fbb.x, k.aa.y - k.fbb.y));
    const float2 n2 = mul2(mul2(G, k.a), k.a);
    const float cI = (k.q.x < 1.0f ? n1.x : n2.x) / d;
    const float cJ = (k.q.y < 1.0f ? n1.y : n2.y) / d;
    gI = k.q.x < 2.0f ? mul2(make_float2(cI, cI), x) : make_float2(0.0f, 0.0f);
    gJ = k.q.y < 2.0f ? mul2(make_float2(cJ, cJ), x) : make_float2(0.0f, 0.0f);
}

// evaluateBoundaryForceWeight(High), WCSPHSolver.cu:66-114 (selected, as above),
// at q = 2d / rad
__device__ __forceinline__ float wall_weight_q(float d, float q, float cs) {
    const float c = 0.02f * cs * cs / (d * d);
    const float r1 = c * 2.0f / 3.0f;
    const float r2 = c * (2.0f * q - 3.0f / 2.0f * q * q);
    const float a = 2.0f - q;
    const float r3 = c * 0.5f * a * a;
    return q < 2.0f / 3.0f ? r1 : (q < 1.0f ? r2 : (q < 2.0f ? r3 : 0.0f));
}

__device__ __forceinline__ float wall_weight(float d, float rad, float cs) {
    return wall_weight_q(d, d * 2.0f / rad, cs);
}

__device__ __forceinline__ float vnorm(float2 v) { return sqrtf(v.x * v.x + v.y * v.y); }

__device__ __forceinline__ float tait(float dens, const Params& P) {
    float a = dens / P.rho0;
    float a3 = a * a * a;
    return P.B * (a3 * a3 * a - 1.0f);
}

// lambda masks indexed by (s_i & 1) << 1 | (s_j & 1); all entries are 0 or 1, so
// they act as predicates (a weight of 1 leaves every product unchanged).
__device__ __forceinline__ bool lamLH(unsigned si, unsigned sj) { return (sj & 1u) == 0u; }        // {1,0,1,0}
__device__ __forceinline__ bool lamHH(unsigned si, unsigned sj) { return !((si & 1u) == 0u && (sj & 1u)); }  // {1,0,1,1}
__device__ __forceinline__ bool lamHL(unsigned si, unsigned sj) { return !((si & 1u) && (sj & 1u)); }        // {1,1,1,0}
__device__ __forceinline__ bool notDeleted(unsigned s) { return s < 2u; }                       // {1,1,0}

// The two terms of a force pair: a for the pressure/viscosity sum, t for the
// sigma sum.
struct PairTerms {
    float2 a, t;
};

// One pair of a force sum: the body of updateAccCell / updateAccCellComplement /
// updateAccCellHigh / updateAccCellComplementHigh (WCSPHSolver.cu:521-558 etc.).
// qi, qj are p/rho^2 of the two particles (the reference's pre/dens2, prej/densj2).
// Both scales' kernels are evaluated as float2 pairs (kern2).  Each sum adds one
// term per pair, so a pair's terms may be evaluated apart from the sums.
__device__ __forceinline__ PairTerms pair_terms(const Params& P, float2 pij, float dist, float2 vij, float qi,
                                                float qj, float densi, float densj, float h) {
    const float2 vp = mul2(vij, pij);
    const float dvp = vp.x + vp.y;
    const float visc = dvp / (dist * dist + 0.01f * h * h) * 2.0f * h * P.alpha * P.cs / (densi + densj);
    float coeff = qi + qj;
    coeff = dvp < 0.0f ? coeff - visc : coeff;  // the reference's `if (dvp < 0) coeff -= ...`
    const Kern2 k = kern2(dist, P);
    float2 gI, gJ;
    kernDW2(k, make_float2(P.GL, P.GH), pij, dist, gI, gJ);
    const float2 w = kernW2(k, make_float2(P.CL, P.CH));
    const float ww = w.x + w.y;
    const float2 half = make_float2(0.5f, 0.5f);  // x / 2 == x * 0.5 exactly
    const float2 g = make_float2(gI.x + gJ.x, gI.y + gJ.y);  // products: added in scalar (see add2)
    return PairTerms{mul2(mul2(make_float2(coeff, coeff), g), half), mul2(mul2(pij, make_float2(ww, ww)), half)};
}

// adds a pair's terms to the force sums (acc, accT) = (s.a, s.t)
__device__ __forceinline__ void add_terms(PairTerms& s, const PairTerms& t) {
    s.a = add2(s.a, t.a);
    s.t = add2(s.t, t.t);
}

// The density term of a pair at distance d: the symmetrised kernel
// (W_r(d) + W_rh(d)) / 2 of computeParticleDensityPressure(High)
// (WCSPHSolver.cu:1342-1516).
__device__ __forceinline__ float pair_density(const Params& P, float d) {
    const float2 w = kernW2(kern2(d, P), make_float2(P.CL, P.CH));
    return (w.x + w.y) / 2.0f;
}

__device__ __forceinline__ float sq(float2 v) {
    const float2 m = mul2(v, v);
    return m.x + m.y;
}

}  // namespace tss
