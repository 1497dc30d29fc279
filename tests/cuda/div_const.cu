// div_const / div_const2 (division by a per-scene constant through its reciprocal
// split, tss_device.cuh) against the IEEE division, bit for bit, on EVERY float a
// with 2^-75 <= |a| <= 2^20 b and on a = +0 (-0, which the kernels never divide,
// may come out +0), for each divisor b: the smoothing lengths of the library's
// workloads, the ends of the accepted radius range [2^-40, 2^40], and 48 seeded
// log-uniform divisors in that range.  The pair kernels divide a = 2d <= 4b, d = 0
// or the square root of a positive float (>= 2^-74.5); the grid coordinates divide
// a position's offset from the origin, whose quotient is a cell coordinate (grids
// of up to 2^20 cells a side are covered).
// Prints "mismatches <count> of <checked>" (and the first mismatch); exits 0
// unless a CUDA call fails.  The kernel touches no memory but two counters.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../../twoscalesplit_gb300/csrc/tss_device.cuh"

using namespace tss;

constexpr unsigned kLo = 52u << 23;  // the bits of 2^-75

// every |a| in [2^-75, hi] (bits kLo..hi, both signs), then a = +0
__global__ void k_check(float b, float yh, float yl, unsigned hi, unsigned long long* bad, unsigned* first) {
    const unsigned long long m = static_cast<unsigned long long>(hi - kLo) + 1ull;
    const unsigned long long n = 2ull * m + 1ull;
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    unsigned long long nbad = 0;
    for (unsigned long long t = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; t < n;
         t += stride) {
        const unsigned u =
            t < 2ull * m ? (kLo + static_cast<unsigned>(t >> 1)) | (static_cast<unsigned>(t & 1ull) << 31) : 0u;
        const float a = __uint_as_float(u);
        const unsigned ref = __float_as_uint(__fdiv_rn(a, b));
        const unsigned s1 = __float_as_uint(div_const(a, b, yh, yl));
        const float2 q2 = div_const2(make_float2(a, a), make_float2(b, b), make_float2(yh, yh), make_float2(yl, yl));
        const bool ok = s1 == ref && __float_as_uint(q2.x) == ref && __float_as_uint(q2.y) == ref;
        if (!ok) {
            ++nbad;
            atomicCAS(first, 0xffffffffu, u);
        }
    }
    if (nbad) atomicAdd(bad, nbad);
}

int main() {
    std::vector<float> bs = {0.001132f, 0.000566f, 0.0667f, 0.03335f, 0.016f, 0.008f, 0.0004f, 0.0002f,
                             1.0f, 3.0f, 0x1p-40f, 0x1p40f, 0.1f, 0.7f, 1e-6f, 12345.678f};
    std::mt19937 rng(7);
    std::uniform_real_distribution<double> u(-40.0, 40.0);
    for (int k = 0; k < 48; ++k) bs.push_back(static_cast<float>(std::exp2(u(rng))));
    unsigned long long* d_bad = nullptr;
    unsigned* d_first = nullptr;
    if (cudaMalloc(&d_bad, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&d_first, sizeof(unsigned)) != cudaSuccess) {
        std::printf("cudaMalloc failed\n");
        return 1;
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    unsigned long long total_bad = 0, checked = 0;
    for (float b : bs) {
        float yh, yl;
        recip_split(b, yh, yl);
        const float lim = std::ldexp(b, 20);
        unsigned hi;
        std::memcpy(&hi, &lim, sizeof(hi));
        cudaMemset(d_bad, 0, sizeof(unsigned long long));
        cudaMemset(d_first, 0xff, sizeof(unsigned));
        k_check<<<sms * 8, 256>>>(b, yh, yl, hi, d_bad, d_first);
        const cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) {
            std::printf("CUDA error: %s\n", cudaGetErrorString(e));
            return 1;
        }
        unsigned long long nb = 0;
        unsigned first = 0;
        cudaMemcpy(&nb, d_bad, sizeof(nb), cudaMemcpyDeviceToHost);
        cudaMemcpy(&first, d_first, sizeof(first), cudaMemcpyDeviceToHost);
        if (nb) {
            float fa;
            std::memcpy(&fa, &first, sizeof(fa));
            std::printf("b=%a: %llu mismatches, first a=%a\n", b, nb, fa);
        }
        total_bad += nb;
        checked += 2ull * (static_cast<unsigned long long>(hi - kLo) + 1ull) + 1ull;
    }
    std::printf("mismatches %llu of %llu\n", total_bad, checked);
    cudaFree(d_bad);
    cudaFree(d_first);
    return 0;
}
