// render.cu -- headless particle splatting into a device RGBA image: the reference's
// display() (TwoScale2D/main.cpp:65-102, 134-138) without OpenGL.
//
// What is restated from the reference's renderers and shaders:
//   * vertex: the particle's normalised device coordinates
//     x = (p.x - xs) / width * 2 - 1 (QuantityRendererVertexShader.glsl:26-27)
//   * geometry: a square of half-size pointSize around it, with relative
//     coordinates -1..1 (QuantityRendererGeometryShader.glsl:35-56)
//   * fragment: discard outside the unit disc; jet colour of the visual quantity
//     (QuantityRendererFragmentShader.glsl:32-54) or a constant colour
//     (PointRendererFragmentShader.glsl:29-34); alpha 0.5
//   * blending: constant colour 0.5, so dst = 0.5 * src + 0.5 * dst per channel,
//     in drawing order (main.cpp:134-138); cleared to (1, 1, 1, 0) (main.cpp:73-74)
//   * visual quantity: min(|rho - rho0|, 400) / 400 (setQuantities, WCSPHSolver.cu:1030-1051)
// A pixel is covered by a splat when its centre's relative coordinates (the
// fragment's interpolated relCoord at that centre) lie in the unit disc.
//
// GPU layout: the image is cut into 16x16 tiles.  Each splat is entered in the list
// of every tile its disc may touch; each tile's list is sorted by splat index in
// shared memory, and each thread of the tile's block blends its pixel through the
// list in that order, so every pixel sees the splats in drawing order and the image
// does not depend on scheduling.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "../../include/tss.h"
#include "solver_impl.cuh"

namespace tss {
namespace {

constexpr int kTile = 16;
constexpr int kSortCap = 4096;   // tile lists up to this size are sorted in shared memory
constexpr int kChunk = 256;      // splats staged per round of the blend loop

struct SplatArgs {
    const float2* pos;
    const float* dens;           // null: constant colour
    const int* n_ptr;            // splats
    const int* nvalid_ptr;       // densities valid below this index (others count as 0), may be null
    float rho0;
    float rgb[3];
    float ps;                    // half-size in normalised device coordinates
    float xs, ys, w, h;          // display rectangle
    int W, H, tx, ty;            // image and tile grid
    unsigned* tile_count;        // [tx*ty] counts, then fill cursors
    int* tile_off;               // [tx*ty + 1]
    int* list;                   // [cap] splat indices by tile
    int cap;
    unsigned* err;
};

__device__ __forceinline__ float ndc_x(const SplatArgs& a, float x) { return (x - a.xs) / a.w * 2.0f - 1.0f; }
__device__ __forceinline__ float ndc_y(const SplatArgs& a, float y) { return (y - a.ys) / a.h * 2.0f - 1.0f; }

// Pixels whose centres may lie within the splat's square, one pixel of margin.
__device__ __forceinline__ bool pixel_box(const SplatArgs& a, float cx, float cy, int& x0, int& x1, int& y0, int& y1) {
    const float fx0 = (cx - a.ps + 1.0f) * 0.5f * a.W - 0.5f, fx1 = (cx + a.ps + 1.0f) * 0.5f * a.W - 0.5f;
    const float fy0 = (cy - a.ps + 1.0f) * 0.5f * a.H - 0.5f, fy1 = (cy + a.ps + 1.0f) * 0.5f * a.H - 0.5f;
    if (!(fx1 >= -1.0f && fx0 <= a.W && fy1 >= -1.0f && fy0 <= a.H)) return false;  // off screen or NaN
    x0 = max(0, static_cast<int>(floorf(fmaxf(fx0, -2.0f))) - 1);
    x1 = min(a.W - 1, static_cast<int>(ceilf(fminf(fx1, a.W + 2.0f))) + 1);
    y0 = max(0, static_cast<int>(floorf(fmaxf(fy0, -2.0f))) - 1);
    y1 = min(a.H - 1, static_cast<int>(ceilf(fminf(fy1, a.H + 2.0f))) + 1);
    return x0 <= x1 && y0 <= y1;
}

__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// getJetColor (QuantityRendererFragmentShader.glsl:32-40)
__device__ __forceinline__ float3 jet(float v) {
    const float f = 4.0f * v;
    return make_float3(clamp01(fminf(f - 1.5f, -f + 4.5f)), clamp01(fminf(f - 0.5f, -f + 3.5f)),
                       clamp01(fminf(f + 0.5f, -f + 2.5f)));
}

__device__ __forceinline__ float3 splat_color(const SplatArgs& a, int i) {
    if (!a.dens) return make_float3(a.rgb[0], a.rgb[1], a.rgb[2]);
    const int nv = a.nvalid_ptr ? *a.nvalid_ptr : *a.n_ptr;
    const float rho = i < nv ? a.dens[i] : 0.0f;
    return jet(fminf(fabsf(rho - a.rho0), 400.0f) / 400.0f);
}

__global__ void k_splat_count(SplatArgs a) {
    const int n = *a.n_ptr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float2 p = a.pos[i];
        int x0, x1, y0, y1;
        if (!pixel_box(a, ndc_x(a, p.x), ndc_y(a, p.y), x0, x1, y0, y1)) continue;
        for (int ty = y0 / kTile; ty <= y1 / kTile; ++ty)
            for (int tx = x0 / kTile; tx <= x1 / kTile; ++tx) atomicAdd(&a.tile_count[ty * a.tx + tx], 1u);
    }
}

// Exclusive scan of the tile counts (one block; the counts become fill cursors).
__global__ void k_splat_scan(SplatArgs a) {
    __shared__ int s_part[1024];
    const int T = a.tx * a.ty;
    const int per = (T + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(T, b + per);
    int sum = 0;
    for (int t = b; t < e; ++t) sum += static_cast<int>(a.tile_count[t]);
    s_part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (unsigned k = 0; k < blockDim.x; ++k) {
            const int v = s_part[k];
            s_part[k] = run;
            run += v;
        }
        a.tile_off[T] = run;
        if (run > a.cap) atomicOr(a.err, kErrCapacity);
    }
    __syncthreads();
    int run = s_part[threadIdx.x];
    for (int t = b; t < e; ++t) {
        const int v = static_cast<int>(a.tile_count[t]);
        a.tile_off[t] = run;
        a.tile_count[t] = 0u;
        run += v;
    }
}

__global__ void k_splat_scatter(SplatArgs a) {
    const int n = *a.n_ptr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float2 p = a.pos[i];
        int x0, x1, y0, y1;
        if (!pixel_box(a, ndc_x(a, p.x), ndc_y(a, p.y), x0, x1, y0, y1)) continue;
        for (int ty = y0 / kTile; ty <= y1 / kTile; ++ty)
            for (int tx = x0 / kTile; tx <= x1 / kTile; ++tx) {
                const int t = ty * a.tx + tx;
                const int k = a.tile_off[t] + static_cast<int>(atomicAdd(&a.tile_count[t], 1u));
                if (k < a.tile_off[t + 1] && k < a.cap) a.list[k] = i;
            }
    }
}

// One block of kTile*kTile threads per tile; each thread owns one pixel.
__global__ void __launch_bounds__(kTile * kTile) k_splat_raster(SplatArgs a, float4* img) {
    __shared__ int s_idx[kSortCap];
    __shared__ float s_cx[kChunk], s_cy[kChunk];
    __shared__ float3 s_col[kChunk];
    const int t = blockIdx.x;
    const int tx = t % a.tx, ty = t / a.tx;
    const int px = tx * kTile + (threadIdx.x % kTile), py = ty * kTile + (threadIdx.x / kTile);
    const bool own = px < a.W && py < a.H;
    float4 c = own ? img[py * a.W + px] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float xp = (static_cast<float>(px) + 0.5f) / static_cast<float>(a.W) * 2.0f - 1.0f;
    const float yp = (static_cast<float>(py) + 0.5f) / static_cast<float>(a.H) * 2.0f - 1.0f;
    const int b = a.tile_off[t], e = min(a.tile_off[t + 1], a.cap);
    const int L = max(0, e - b);
    // the tile's splats in drawing order: a bitonic sort of the list in shared
    // memory, or (lists beyond kSortCap) repeated selection of the next index
    const bool small = L <= kSortCap;
    int P = 1;
    while (P < L) P <<= 1;
    if (small) {
        for (int k = threadIdx.x; k < P; k += blockDim.x) s_idx[k] = k < L ? a.list[b + k] : 0x7fffffff;
        __syncthreads();
        for (int size = 2; size <= P; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int k = threadIdx.x; k < P; k += blockDim.x) {
                    const int m = k ^ stride;
                    if (m > k) {
                        const bool up = (k & size) == 0;
                        const int u = s_idx[k], v = s_idx[m];
                        if ((u > v) == up) {
                            s_idx[k] = v;
                            s_idx[m] = u;
                        }
                    }
                }
                __syncthreads();
            }
    }
    __shared__ int s_last, s_next;
    if (threadIdx.x == 0) s_last = -1;
    __syncthreads();
    for (int base = 0; base < L; base += kChunk) {
        const int m = min(kChunk, L - base);
        if (small) {
            for (int k = threadIdx.x; k < m; k += blockDim.x) {
                const int i = s_idx[base + k];
                const float2 p = a.pos[i];
                s_cx[k] = ndc_x(a, p.x);
                s_cy[k] = ndc_y(a, p.y);
                s_col[k] = splat_color(a, i);
            }
        } else {
            for (int k = 0; k < m; ++k) {  // selection: the smallest index above the last one taken
                if (threadIdx.x == 0) s_next = 0x7fffffff;
                __syncthreads();
                int best = 0x7fffffff;
                for (int q = threadIdx.x; q < L; q += blockDim.x) {
                    const int v = a.list[b + q];
                    if (v > s_last && v < best) best = v;
                }
                atomicMin(&s_next, best);
                __syncthreads();
                if (threadIdx.x == 0) {
                    const int i = s_next;
                    s_last = i;
                    const float2 p = a.pos[i];
                    s_cx[k] = ndc_x(a, p.x);
                    s_cy[k] = ndc_y(a, p.y);
                    s_col[k] = splat_color(a, i);
                }
                __syncthreads();
            }
        }
        __syncthreads();
        if (own) {
            for (int k = 0; k < m; ++k) {
                const float rx = (xp - s_cx[k]) / a.ps, ry = (yp - s_cy[k]) / a.ps;
                if (rx * rx + ry * ry <= 1.0f) {  // inside the disc (no discard)
                    c.x = 0.5f * s_col[k].x + 0.5f * c.x;
                    c.y = 0.5f * s_col[k].y + 0.5f * c.y;
                    c.z = 0.5f * s_col[k].z + 0.5f * c.z;
                    c.w = 0.5f * 0.5f + 0.5f * c.w;
                }
            }
        }
        __syncthreads();
    }
    if (own) img[py * a.W + px] = c;
}

__global__ void k_clear(float4* img, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        img[i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
}

size_t ws_size(int cap, int W, int H) {
    const size_t T = static_cast<size_t>((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile);
    return al256(sizeof(unsigned) * T) + al256(sizeof(int) * (T + 1)) + al256(sizeof(int) * static_cast<size_t>(cap)) +
           256;
}

bool view_ok(const tss_view* v) {
    return v && v->width > 0 && v->height > 0 && v->width <= 16384 && v->height <= 16384 && v->xe > v->xs &&
           v->ye > v->ys;
}

// Splat entries a render may need: each splat touches at most the tiles of its box.
int entries_cap(int n, const tss_view* v, float ps) {
    const double span = std::floor((static_cast<double>(ps) * std::max(v->width, v->height) + 6.0) / kTile) + 2.0;
    const double per = span * span;
    const double cap = static_cast<double>(n) * per + 1024.0;
    return cap > 2.0e9 ? 2000000000 : static_cast<int>(cap);
}

// Enqueue one splat pass (count, scan, scatter, raster) over device counts.
cudaError_t splat_enqueue(const tss_view* v, const float2* pos, const float* dens, const int* n_ptr,
                          const int* nvalid_ptr, int n_cap, float rho0, const float rgb[3], float ps, float4* img,
                          char* ws, int cap, unsigned* err, cudaStream_t st) {
    SplatArgs a{};
    a.pos = pos;
    a.dens = dens;
    a.n_ptr = n_ptr;
    a.nvalid_ptr = nvalid_ptr;
    a.rho0 = rho0;
    for (int k = 0; k < 3; ++k) a.rgb[k] = rgb ? rgb[k] : 0.0f;
    a.ps = ps;
    a.xs = v->xs;
    a.ys = v->ys;
    a.w = v->xe - v->xs;  // Rectangle::GetWidth
    a.h = v->ye - v->ys;
    a.W = v->width;
    a.H = v->height;
    a.tx = (v->width + kTile - 1) / kTile;
    a.ty = (v->height + kTile - 1) / kTile;
    const size_t T = static_cast<size_t>(a.tx) * a.ty;
    a.tile_count = reinterpret_cast<unsigned*>(ws);
    a.tile_off = reinterpret_cast<int*>(ws + al256(sizeof(unsigned) * T));
    a.list = reinterpret_cast<int*>(ws + al256(sizeof(unsigned) * T) + al256(sizeof(int) * (T + 1)));
    a.cap = cap;
    a.err = err;
    cudaError_t e = cudaMemsetAsync(a.tile_count, 0, sizeof(unsigned) * T, st);
    if (e != cudaSuccess) return e;
    const int pb = particle_blocks(n_cap > 0 ? n_cap : 1, 256);
    k_splat_count<<<pb, 256, 0, st>>>(a);
    k_splat_scan<<<1, 1024, 0, st>>>(a);
    k_splat_scatter<<<pb, 256, 0, st>>>(a);
    k_splat_raster<<<static_cast<unsigned>(T), kTile * kTile, 0, st>>>(a, img);
    return cudaGetLastError();
}

}  // namespace
}  // namespace tss

using namespace tss;

extern "C" {

tss_status tss_render_workspace_size(int n, const tss_view* v, float point_size, size_t* bytes) {
    if (!bytes || n < 0 || !view_ok(v) || !(point_size > 0.0f)) return TSS_INVALID_ARG;
    *bytes = ws_size(entries_cap(n, v, point_size), v->width, v->height) + 256;
    return TSS_OK;
}

tss_status tss_render_clear(float* d_rgba, int width, int height, void* stream) {
    if (!d_rgba || width <= 0 || height <= 0) return TSS_INVALID_ARG;
    const int n = width * height;
    k_clear<<<particle_blocks(n, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(reinterpret_cast<float4*>(d_rgba), n);
    return cudaGetLastError() == cudaSuccess ? TSS_OK : TSS_CUDA_ERROR;
}

tss_status tss_render_splats(const tss_view* v, int n, const float* d_pos, const float* d_dens, float rest_density,
                             const float* rgb, float point_size, float* d_rgba, void* d_workspace,
                             size_t workspace_bytes, void* stream) {
    if (!view_ok(v) || n < 0 || (n > 0 && !d_pos) || !d_rgba || !d_workspace || !(point_size > 0.0f) ||
        (!d_dens && !rgb))
        return TSS_INVALID_ARG;
    size_t need = 0;
    if (tss_render_workspace_size(n, v, point_size, &need) != TSS_OK || workspace_bytes < need) return TSS_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    char* w = static_cast<char*>(d_workspace);
    int* n_dev = reinterpret_cast<int*>(w);
    unsigned* err = reinterpret_cast<unsigned*>(w + 64);
    if (cudaMemsetAsync(w, 0, 256, st) != cudaSuccess) return TSS_CUDA_ERROR;
    k_set_int<<<1, 1, 0, st>>>(n_dev, n);
    const cudaError_t e = splat_enqueue(v, reinterpret_cast<const float2*>(d_pos), d_dens, n_dev, nullptr, n,
                                        rest_density, rgb, point_size, reinterpret_cast<float4*>(d_rgba), w + 256,
                                        entries_cap(n, v, point_size), err, st);
    return e == cudaSuccess ? TSS_OK : TSS_CUDA_ERROR;
}

// display(): white clear, low-res splats (jet), high-res splats (jet), walls (black).
tss_status tss_solver_render(tss_solver* s, const tss_view* v, const float* point_sizes, float* d_rgba, void* stream) {
    if (!s || !view_ok(v) || !point_sizes || !d_rgba || s->batched) return TSS_INVALID_ARG;
    for (int k = 0; k < 3; ++k)
        if (!(point_sizes[k] > 0.0f)) return TSS_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int caps[3] = {s->nL, s->capH, s->nW};
    size_t need = 0;
    for (int k = 0; k < 3; ++k) need = std::max(need, ws_size(entries_cap(caps[k], v, point_sizes[k]), v->width, v->height));
    need += 256;
    cudaError_t e = s->enter(st);
    if (e != cudaSuccess) return s->cuda_fail(e, "render");
    if (need > s->render_ws_bytes) {
        if ((e = s->wait_idle()) != cudaSuccess) return s->cuda_fail(e, "render");
        if (s->render_ws) cudaFree(s->render_ws);
        s->render_ws = nullptr;
        s->render_ws_bytes = 0;
        if ((e = cudaMalloc(&s->render_ws, need)) != cudaSuccess) return s->cuda_fail(e, "render workspace");
        s->render_ws_bytes = need;
    }
    char* w = static_cast<char*>(s->render_ws);
    int* nw = reinterpret_cast<int*>(w);
    unsigned* err = &s->cnt->err;
    const float black[3] = {0.0f, 0.0f, 0.0f};
    if (tss_render_clear(d_rgba, v->width, v->height, stream) != TSS_OK) return TSS_CUDA_ERROR;
    k_set_int<<<1, 1, 0, st>>>(nw, s->nW);
    const float rho0 = s->P.rho0;
    float4* img = reinterpret_cast<float4*>(d_rgba);
    // densities of the last step are valid for the list entries it sorted
    const int* valid[2] = {s->carry ? nullptr : &s->cnt->sorted[0], s->carry ? nullptr : &s->cnt->sorted[1]};
    const float* dens[2] = {s->carry ? s->L.ndens : s->L.dens, s->carry ? s->H.ndens : s->H.dens};
    e = splat_enqueue(v, s->L.npos, dens[0], &s->cnt->cur[0], valid[0], s->nL, rho0, nullptr,
                                  point_sizes[0], img, w + 256, entries_cap(caps[0], v, point_sizes[0]), err, st);
    if (e == cudaSuccess)
        e = splat_enqueue(v, s->H.npos, dens[1], &s->cnt->cur[1], valid[1], s->capH, rho0, nullptr, point_sizes[1], img,
                          w + 256, entries_cap(caps[1], v, point_sizes[1]), err, st);
    if (e == cudaSuccess && s->nW > 0)
        e = splat_enqueue(v, s->wpos, nullptr, nw, nullptr, s->nW, rho0, black, point_sizes[2], img, w + 256,
                          entries_cap(caps[2], v, point_sizes[2]), err, st);
    if (e == cudaSuccess) e = s->leave(st);
    if (e != cudaSuccess) return s->cuda_fail(e, "render");
    return TSS_OK;
}

}  // extern "C"
