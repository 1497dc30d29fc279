// cuda_shim.h -- lets the reference's CUDA kernel source compile as plain C++ so
// that its kernels can be run on the CPU, one thread index at a time.  Part of the
// ORACLE (test infrastructure): it is used only to pin the CPU restatement
// (tss_oracle.cpp) against the reference's own code.
//
// What it maps:
//  * __device__/__global__/__constant__/__shared__ -> ordinary C++
//  * blockIdx/threadIdx/blockDim                     -> globals set by the harness
//  * __syncthreads()                                 -> two-phase emulation: in phase
//    0 a thread returns at the barrier, in phase 1 it re-runs the (idempotent)
//    pre-barrier part and continues (valid for the one kernel that uses it,
//    computeCellStartEndIndices, WCSPHSolver.cu:1300-1340)
//  * atomicAdd                                       -> sequential read-modify-write
//  * texture<> / tex1Dfetch                          -> bounded pointer reads that
//    return 0 out of range, as a 1D texture fetch does (WCSPHSolver.cu:1938-1939
//    fetch past the bound range)
//  * float2 / int2                                   -> zero-initialised structs, so
//    the uninitialised accumulator of WCSPHSolver.cu:1919 starts at zero
//  * min/max/abs/sqrt/exp overloads as CUDA's device math headers provide them;
//    min(float, double) promotes to double like CUDA's mixed overload.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>

#define __device__
#define __global__
#define __constant__
#define __shared__
#define __host__

struct shim_uint3 {
    unsigned int x, y, z;
};
extern shim_uint3 blockIdx, threadIdx, blockDim, gridDim;
extern int g_shim_phase;
#define __syncthreads()          \
    do {                         \
        if (g_shim_phase == 0) { \
            return;              \
        }                        \
    } while (0)

struct float2 {
    float x, y;
    float2() : x(0.f), y(0.f) {}
};
struct int2 {
    int x, y;
    int2() : x(0), y(0) {}
};

enum { cudaTextureType1D = 1 };
enum { cudaReadModeElementType = 0 };
template <class T, int Dim, int Mode>
struct texture {
    const T* ptr = nullptr;
    long n = 0;
};
template <class T, int D, int M>
inline T tex1Dfetch(const texture<T, D, M>& t, int i) {
    return (i >= 0 && i < t.n) ? t.ptr[i] : T(0);
}

inline int atomicAdd(int* p, int v) {
    int o = *p;
    *p += v;
    return o;
}

inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline float min(float a, float b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline double min(float a, double b) { return std::fmin(static_cast<double>(a), b); }
using std::abs;
using std::exp;
using std::sqrt;
