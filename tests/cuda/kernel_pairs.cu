// Packed kernel pairs against the scalar kernels: kern2 / kernW2 / kernDW2 (both
// scales in float2 pairs) must give the bits of kernW / kernDW, one scale at a time,
// for every distance.  The packed forms rely on the compiler not contracting a
// packed product into a following add (tss_device.cuh); this checks that on random
// distances in [0, r] for the radius given on the command line.
// Prints "mismatches <count> of <n>"; exits 0 unless a CUDA call fails.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "../../twoscalesplit_gb300/csrc/tss_device.cuh"

using namespace tss;

__global__ void k_pairs(const float* d, const float2* x, int n, Params P, float* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float di = d[i];
    const float2 xi = x[i];
    float* o = out + 12 * static_cast<size_t>(i);
    const float2 gr = kernDW(xi, di, P.r, P.GL), gh = kernDW(xi, di, P.rh, P.GH);
    o[0] = kernW(di, P.r, P.CL);
    o[1] = kernW(di, P.rh, P.CH);
    o[2] = gr.x;
    o[3] = gr.y;
    o[4] = gh.x;
    o[5] = gh.y;
    const Kern2 k = kern2(di, P);
    const float2 w = kernW2(k, make_float2(P.CL, P.CH));
    float2 gI, gJ;
    kernDW2(k, make_float2(P.GL, P.GH), xi, di, gI, gJ);
    o[6] = w.x;
    o[7] = w.y;
    o[8] = gI.x;
    o[9] = gI.y;
    o[10] = gJ.x;
    o[11] = gJ.y;
}

int main(int argc, char** argv) {
    const int n = 1 << 22;
    Params P{};
    P.r = argc > 1 ? static_cast<float>(atof(argv[1])) : 0.001132f;
    P.rh = P.r * 0.5f;
    const double pi = 3.14159265358979323846;
    P.CL = static_cast<float>(10.0 / (7.0 * pi * P.r * P.r));
    P.CH = static_cast<float>(10.0 / (7.0 * pi * P.rh * P.rh));
    P.GL = static_cast<float>(-30.0 / (7.0 * pi * P.r * P.r * P.r));
    recip_split(P.r, P.inv_hi.x, P.inv_lo.x);
    recip_split(P.rh, P.inv_hi.y, P.inv_lo.y);
    P.GH = static_cast<float>(-30.0 / (7.0 * pi * P.rh * P.rh * P.rh));
    std::mt19937 rng(1);
    std::uniform_real_distribution<float> u(0.0f, 1.0f);
    std::vector<float> d(n);
    std::vector<float2> x(n);
    for (int i = 0; i < n; ++i) {
        d[i] = u(rng) * P.r;
        x[i] = make_float2((u(rng) - 0.5f) * P.r, (u(rng) - 0.5f) * P.r);
    }
    float *dd = nullptr, *dout = nullptr;
    float2* dx = nullptr;
    if (cudaMalloc(&dd, sizeof(float) * n) != cudaSuccess || cudaMalloc(&dx, sizeof(float2) * n) != cudaSuccess ||
        cudaMalloc(&dout, sizeof(float) * 12 * static_cast<size_t>(n)) != cudaSuccess) {
        std::printf("cudaMalloc failed\n");
        return 1;
    }
    cudaMemcpy(dd, d.data(), sizeof(float) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(dx, x.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
    k_pairs<<<(n + 255) / 256, 256>>>(dd, dx, n, P, dout);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        std::printf("CUDA error: %s\n", cudaGetErrorString(e));
        return 1;
    }
    std::vector<float> o(12 * static_cast<size_t>(n));
    cudaMemcpy(o.data(), dout, sizeof(float) * o.size(), cudaMemcpyDeviceToHost);
    long bad = 0;
    for (int i = 0; i < n; ++i)
        if (std::memcmp(&o[12 * static_cast<size_t>(i)], &o[12 * static_cast<size_t>(i) + 6], 6 * sizeof(float)))
            ++bad;
    std::printf("mismatches %ld of %d\n", bad, n);
    cudaFree(dd);
    cudaFree(dx);
    cudaFree(dout);
    return 0;
}
