// refgpu_shim.cuh -- prologue for compiling the reference's kernel source
// (TwoScale2D/WCSPHSolver.cu, constants, device functions and kernels) for sm_103a
// as it stands, so that its own kernels can be timed on this GPU beside this
// library.  Part of the ORACLE (test and measurement infrastructure).
//
// What it maps:
//  * texture<T, 1D, ElementType> references (removed from CUDA 12): a __device__
//    struct with the bound pointer and element count; tex1Dfetch returns 0 outside
//    the bound range, as a 1D texture fetch does (WCSPHSolver.cu:1938-1939 fetch
//    past it).  The launcher fills the structs where Bind() bound the textures.
//  * __global__: the kernels are compiled as __device__ functions; the entry
//    kernels after the source (refgpu_entry.inc, extern "C" names the launcher can
//    look up) call them with the launch's own thread indices.
#pragma once
#include <cuda_runtime.h>

template <class T, int Dim, int Mode>
struct ref_tex {
    const T* ptr;
    int n;
};

template <class T, int Dim, int Mode>
__device__ __forceinline__ T tex1Dfetch(const ref_tex<T, Dim, Mode>& t, int i) {
    return (i >= 0 && i < t.n) ? t.ptr[i] : T(0);
}

#define texture __device__ ref_tex
#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
