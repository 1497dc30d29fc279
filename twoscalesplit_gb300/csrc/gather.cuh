// gather.cuh -- the two ways a gather walks one particle's cell window.
//
// PerThread: one particle per thread, 32 particles per warp.  Each thread walks its
// window's rows in order, testing each candidate and evaluating an accepted pair
// at once.  This is the throughput form: consecutive threads walk overlapping
// windows, so neighbour loads are shared through L1.  (A cursor that searched on
// to the next accepted candidate before evaluating, so that a warp's lanes met at
// the pair arithmetic, was 4-8 % slower in the density gathers and no faster in
// the force gathers on a developed 1M-particle dam break.)
//
// PerWarp: one particle per warp.  The 32 lanes test 32 consecutive candidates of
// a row at a time and evaluate the accepted pairs' terms in parallel; then every
// lane adds the terms in candidate order, taking each from the lane that evaluated
// it (warp shuffles), so every lane ends with the per-thread sum, bit for bit.  For
// scenes too small to fill the GPU, where a step is bound by each thread's chain
// of dependent loads rather than by instruction issue.
//
// A gather is written once against the policy G: G::window / G::window_if /
// G::span take the candidate test (which may leave state for the term: the
// per-thread walk evaluates a candidate's term right after its test), the pair
// term, the accumulation, and the running sum.  Per-particle results are stored
// by G::leader() only.
#pragma once
#include "tss_device.cuh"

namespace tss {

__device__ __forceinline__ float shfl_from(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float2 shfl_from(float2 v, int src) {
    return make_float2(shfl_from(v.x, src), shfl_from(v.y, src));
}
__device__ __forceinline__ PairTerms shfl_from(const PairTerms& v, int src) {
    return PairTerms{shfl_from(v.a, src), shfl_from(v.t, src)};
}

struct PerThread {
    static constexpr bool kWarp = false;
    __device__ __forceinline__ static bool leader() { return true; }

    template <class T, class Test, class Term, class Add>
    __device__ __forceinline__ static void window(const int* off, int dimx, int csx, int cex, int csy, int cey,
                                                  Test&& test, Term&& term, Add&& add, T& sum) {
        for (int cy = csy; cy <= cey; ++cy) {
            const int row = cy * dimx;
            span(off[row + csx], off[row + cex + 1], test, term, add, sum);
        }
    }

    // the candidates [a, b), in order
    template <class T, class Test, class Term, class Add>
    __device__ __forceinline__ static void span(int a, int b, Test&& test, Term&& term, Add&& add, T& sum) {
        for (int k = a; k < b; ++k)
            if (test(k)) add(sum, term(k));
    }

    // window() for a walk whose test is a key of the candidate alone: key(k) (a
    // float, e.g. the squared distance), ok(x) the test on it, term(k, x).  U (2 or
    // 4) candidates per trip: their keys are formed before any of their terms is
    // evaluated, in candidate order, which cuts the loop's own instructions and
    // keeps U neighbour loads in flight.  On a developed 1M-particle dam break, two
    // per trip took 3-7 % off the densities against one; four took 4-5 % more off
    // the high-res density (whose key also loads the candidate's state) and was
    // 2-3 % slower than two in the low-res density.
    template <int U, class T, class Key, class Ok, class Term, class Add>
    __device__ __forceinline__ static void window_keyed(const int* off, int dimx, int csx, int cex, int csy, int cey,
                                                        Key&& key, Ok&& ok, Term&& term, Add&& add, T& sum) {
        static_assert(U == 2 || U == 4, "two or four candidates per trip");
        for (int cy = csy; cy <= cey; ++cy) {
            const int row = cy * dimx;
            const int b = off[row + cex + 1];
            int k = off[row + csx];
            if constexpr (U == 4) {
                for (; k + 3 < b; k += 4) {
                    const float x0 = key(k), x1 = key(k + 1), x2 = key(k + 2), x3 = key(k + 3);
                    if (ok(x0)) add(sum, term(k, x0));
                    if (ok(x1)) add(sum, term(k + 1, x1));
                    if (ok(x2)) add(sum, term(k + 2, x2));
                    if (ok(x3)) add(sum, term(k + 3, x3));
                }
            }
            for (; k + 1 < b; k += 2) {
                const float x0 = key(k), x1 = key(k + 1);
                if (ok(x0)) add(sum, term(k, x0));
                if (ok(x1)) add(sum, term(k + 1, x1));
            }
            if (k < b) {
                const float x0 = key(k);
                if (ok(x0)) add(sum, term(k, x0));
            }
        }
    }

    // window() over the rows for which live(row) holds (row = cy * dimx).  A row
    // left out must hold no candidate that passes the test: the sum is the same.
    template <class T, class Live, class Test, class Term, class Add>
    __device__ __forceinline__ static void window_if(const int* off, int dimx, int csx, int cex, int csy, int cey,
                                                     Live&& live, Test&& test, Term&& term, Add&& add, T& sum) {
        for (int cy = csy; cy <= cey; ++cy) {
            const int row = cy * dimx;
            if (live(row)) span(off[row + csx], off[row + cex + 1], test, term, add, sum);
        }
    }
};

struct PerWarp {
    static constexpr bool kWarp = true;
    __device__ __forceinline__ static bool leader() { return (threadIdx.x & 31u) == 0u; }

    // a and b are the same in every lane (one particle per warp)
    template <class T, class Test, class Term, class Add>
    __device__ __forceinline__ static void span(int a, int b, Test&& test, Term&& term, Add&& add, T& sum) {
        const int lane = static_cast<int>(threadIdx.x & 31u);
        for (int base = a; base < b; base += 32) {
            const int k = base + lane;
            T t{};
            const bool ok = k < b && test(k);
            if (ok) t = term(k);
            unsigned m = __ballot_sync(0xffffffffu, ok);
            while (m) {  // the accepted candidates in order: lane order is candidate order
                const int src = __ffs(m) - 1;
                m &= m - 1u;
                add(sum, shfl_from(t, src));
            }
        }
    }

    template <class T, class Test, class Term, class Add>
    __device__ __forceinline__ static void window(const int* off, int dimx, int csx, int cex, int csy, int cey,
                                                  Test&& test, Term&& term, Add&& add, T& sum) {
        for (int cy = csy; cy <= cey; ++cy) {
            const int row = cy * dimx;
            span(off[row + csx], off[row + cex + 1], test, term, add, sum);
        }
    }

    template <int U, class T, class Key, class Ok, class Term, class Add>
    __device__ __forceinline__ static void window_keyed(const int* off, int dimx, int csx, int cex, int csy, int cey,
                                                        Key&& key, Ok&& ok, Term&& term, Add&& add, T& sum) {
        float x = 0.0f;
        window(
            off, dimx, csx, cex, csy, cey,
            [&](int k) {
                x = key(k);
                return ok(x);
            },
            [&](int k) { return term(k, x); }, add, sum);
    }

    // live(row) is the same in every lane (one particle per warp)
    template <class T, class Live, class Test, class Term, class Add>
    __device__ __forceinline__ static void window_if(const int* off, int dimx, int csx, int cex, int csy, int cey,
                                                     Live&& live, Test&& test, Term&& term, Add&& add, T& sum) {
        for (int cy = csy; cy <= cey; ++cy) {
            const int row = cy * dimx;
            if (live(row)) span(off[row + csx], off[row + cex + 1], test, term, add, sum);
        }
    }
};

}  // namespace tss
