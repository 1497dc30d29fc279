// grid.cu -- counting-sort grid build (see grid.cuh) and the tss_grid_build entry
// point of the C ABI.
#include <cuda_runtime.h>

#include "../../include/tss.h"
#include "grid.cuh"

namespace tss {

int sm_count() {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 152;
    }
    return sms;
}

int particle_blocks(int cap, int threads) {
    long long need = (static_cast<long long>(cap) + threads - 1) / threads;
    long long lim = static_cast<long long>(sm_count()) * 16;
    long long b = need < lim ? need : lim;
    return b < 1 ? 1 : static_cast<int>(b);
}

__global__ void k_grid_keys(const float2* __restrict__ pos, const int* __restrict__ n_ptr, float ox, float oy,
                            float cell, int dimx, int dimy, unsigned* __restrict__ count, int* __restrict__ key,
                            int* __restrict__ rank, unsigned* __restrict__ tile_sum) {
    const int n = *n_ptr;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        grid_key(count, key, rank, tile_sum, i, cell_hash(pos[i], ox, oy, cell, dimx, dimy));
}

// Tiles of kScanTile counts, strided over the blocks.  A tile's offset is the sum
// of the tile sums before it (read from L2), so tiles are independent and nothing
// waits on another block.  Only the cells in use are scanned (a pool's grids are
// sized for its capacity); counts are zeroed for the next key pass (only the
// 16-byte groups that hold a non-zero count are written back).
__global__ void __launch_bounds__(kScanThreads) k_grid_scan(GridBufs g) {
    __shared__ unsigned s_warp[kScanThreads / 32];
    __shared__ unsigned s_red[kScanThreads / 32];
    const int C = g.used ? min(*g.used, g.ncells) : g.ncells;
    const int ntiles = (C + kScanTile - 1) / kScanTile;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (C <= 0) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            g.off[0] = 0;
            *g.total = 0;
        }
        return;
    }
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        unsigned before = 0;
        for (int t = threadIdx.x; t < tile; t += blockDim.x) before += g.tile_sum[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
        if (lane == 0) s_red[warp] = before;
        const int base = tile * kScanTile + threadIdx.x * kScanItems;
        unsigned v[kScanItems];
        const bool full = base + kScanItems <= C;
        if (full) {
            uint4* p = reinterpret_cast<uint4*>(g.count + base);
#pragma unroll
            for (int q = 0; q < kScanItems / 4; ++q) {
                const uint4 a = p[q];
                v[4 * q] = a.x;
                v[4 * q + 1] = a.y;
                v[4 * q + 2] = a.z;
                v[4 * q + 3] = a.w;
                if (a.x | a.y | a.z | a.w) p[q] = make_uint4(0, 0, 0, 0);
            }
        } else {
#pragma unroll
            for (int k = 0; k < kScanItems; ++k) {
                int idx = base + k;
                v[k] = idx < C ? g.count[idx] : 0u;
                if (idx < C && v[k]) g.count[idx] = 0u;
            }
        }
        unsigned sum = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            sum += v[k];
            if (v[k] > static_cast<unsigned>(kBigCell)) {  // ordered by a block sort in the reorder
                const int slot = atomicAdd(g.nbig, 1);
                if (slot < g.big_cap) g.big[slot] = base + k;
            }
        }
        unsigned inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            unsigned w = lane < kScanThreads / 32 ? s_warp[lane] : 0u;
            unsigned r = lane < kScanThreads / 32 ? s_red[lane] : 0u;
            unsigned wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                unsigned t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
            if (lane < kScanThreads / 32) s_warp[lane] = wi - w + r;  // exclusive warp offsets + tile prefix
        }
        __syncthreads();
        unsigned run = s_warp[warp] + (inc - sum);
        if (full) {
            int4* q = reinterpret_cast<int4*>(g.off + base);
#pragma unroll
            for (int k = 0; k < kScanItems / 4; ++k) {
                int4 o4;
                o4.x = static_cast<int>(run);
                run += v[4 * k];
                o4.y = static_cast<int>(run);
                run += v[4 * k + 1];
                o4.z = static_cast<int>(run);
                run += v[4 * k + 2];
                o4.w = static_cast<int>(run);
                run += v[4 * k + 3];
                q[k] = o4;
            }
            if (base + kScanItems == C) {
                g.off[C] = static_cast<int>(run);
                *g.total = static_cast<int>(run);
            }
        } else {
#pragma unroll
            for (int k = 0; k < kScanItems; ++k) {
                int idx = base + k;
                if (idx < C) g.off[idx] = static_cast<int>(run);
                run += v[k];
                if (idx == C - 1) {
                    g.off[C] = static_cast<int>(run);
                    *g.total = static_cast<int>(run);
                }
            }
        }
        __syncthreads();  // s_warp / s_red are reused by the next tile
    }
}

// Every index below is checked: offsets that do not fit the keys or ranks (a
// caller's table, ids that are not distinct) set kErrGridIndex, and the build then
// skips those entries instead of touching memory outside its buffers.
__global__ void k_grid_scatter(const int* __restrict__ n_ptr, const int32_t* __restrict__ id, GridBufs g,
                               unsigned* err) {
    const int n = *n_ptr;
    const int total = *g.total;
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the scan's list of big cells, for the reorder
        *g.nbig_snap = *g.nbig;
        *g.nbig = 0;  // empty for the next build's scan
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int c = g.key[i];
        if (c < 0) continue;  // dropped from the list
        if (c >= g.ncells) {
            atomicOr(err, kErrGridIndex);
            continue;
        }
        const int dst = g.off[c] + g.rank[i];
        if (dst < 0 || dst >= total) {
            atomicOr(err, kErrGridIndex);
            continue;
        }
        g.perm[dst] = make_int2(i, id[i]);
    }
}

namespace {

// Gathers list entry src's state into sorted position dst.
__device__ __forceinline__ void reorder_move(const ReorderArgs& a, int src, int dst, int id, unsigned* err) {
    if (a.dst_pos) a.dst_pos[dst] = a.src_pos[src];
    if (a.src_vel) a.dst_vel[dst] = a.src_vel[src];
    if (a.src_st) {
        uint8_t st = a.src_st[src];
        a.dst_st[dst] = st;
        if (a.h_state0 && (st & 1u) == 0u) *a.h_state0 = 1;
    }
    if (a.dst_id) a.dst_id[dst] = id;
    if (a.src_dens) {
        a.dst_dens[dst] = a.src_dens[src];
        a.dst_pres[dst] = a.src_pres[src];
    }
    if (a.dst_order) a.dst_order[dst] = src;
    if (a.dst_sc) a.dst_sc[dst] = a.page_scene[(id >> a.id_shift) >> a.page_shift];
    if (a.slot_map) {
        if (id >= 0 && id < a.slots) a.slot_map[id] = dst;
        else atomicOr(err, kErrGridIndex);
    }
}

// Sorts the ids of k entries (perm[0..k).y, non-negative) ascending with the whole
// block (kReorderThreads threads): least-significant-digit radix sort, 8-bit
// digits, as many passes as the largest id needs, between buffers x and y (k ints
// each, global memory).  Each pass is a block histogram, its exclusive scan, and a
// stable scatter of the entries in tiles of kReorderThreads, taken in order: an
// entry's place is its digit's running base + the same-digit entries of earlier
// warps in the tile + its rank among its warp's same-digit lanes.  Returns the
// buffer holding the sorted ids.  Every thread of the block must call it.
__device__ const int* block_sort_ids(const int2* __restrict__ perm, int k, int* x, int* y) {
    constexpr int kWarps = kReorderThreads / 32;
    __shared__ unsigned s_base[256];
    __shared__ unsigned s_wcnt[kWarps][256];
    __shared__ unsigned s_max[kWarps];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned mx = 0;
    for (int i = t; i < k; i += kReorderThreads) {
        const int id = perm[i].y;
        x[i] = id;
        mx = max(mx, static_cast<unsigned>(id));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s_max[warp] = mx;
    for (int w = 0; w < kWarps; ++w) s_wcnt[w][t] = 0u;
    __syncthreads();
    mx = 0;
    for (int w = 0; w < kWarps; ++w) mx = max(mx, s_max[w]);
    const int bits = 32 - __clz(static_cast<int>(mx | 1u));
    const int passes = (bits + 7) / 8;
    const unsigned lt = (1u << lane) - 1u;
    int* in = x;
    int* out = y;
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = 8 * pass;
        s_base[t] = 0u;
        __syncthreads();
        for (int i = t; i < k; i += kReorderThreads) atomicAdd(&s_base[(in[i] >> shift) & 255], 1u);
        __syncthreads();
        // exclusive scan of the 256 digit counts (one per thread)
        const unsigned c = s_base[t];
        unsigned inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        if (lane == 31) s_max[warp] = inc;
        __syncthreads();
        unsigned before = 0;
        for (int w = 0; w < warp; ++w) before += s_max[w];
        s_base[t] = before + inc - c;
        __syncthreads();
        for (int t0 = 0; t0 < k; t0 += kReorderThreads) {
            const int i = t0 + t;
            const bool valid = i < k;
            const int v = valid ? in[i] : 0;
            const unsigned dg = static_cast<unsigned>(v >> shift) & 255u;
            // lanes past k take keys no digit has, so they group with nothing
            const unsigned peers = __match_any_sync(0xffffffffu, valid ? dg : 256u + lane);
            const unsigned r = __popc(peers & lt);
            if (valid && r == 0) s_wcnt[warp][dg] = __popc(peers);
            __syncthreads();
            if (valid) {
                unsigned dst = s_base[dg] + r;
                for (int w = 0; w < warp; ++w) dst += s_wcnt[w][dg];
                out[dst] = v;
            }
            __syncthreads();
            unsigned sum = 0;
            for (int w = 0; w < kWarps; ++w) {
                sum += s_wcnt[w][t];
                s_wcnt[w][t] = 0u;
            }
            s_base[t] += sum;
            __syncthreads();
        }
        int* tmp = in;
        in = out;
        out = tmp;
    }
    return in;
}

// the number of entries of sorted[0..k) below id
__device__ __forceinline__ int lower_rank(const int* __restrict__ sorted, int k, int id) {
    int lo = 0, hi = k;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (sorted[mid] < id) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

}  // namespace

// The sorted entries are [0, total); the list count *n_ptr becomes total (only
// block 0 writes it, and nothing in this kernel reads it).  Entries of cells with
// at most kBigCell entries are placed by counting the smaller ids of their cell;
// the bigger cells (listed by the scan) are placed whole by one block each.
__global__ void __launch_bounds__(kReorderThreads) k_grid_reorder(int* n_ptr, int cap, GridBufs g, ReorderArgs a,
                                                                  unsigned* err) {
    const int n = *g.total;
    if (blockIdx.x == 0 && threadIdx.x == 0) *n_ptr = n;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int2 pe = g.perm[k];
        const int src = pe.x, id = pe.y;
        if (src < 0 || src >= cap) {
            atomicOr(err, kErrGridIndex);
            continue;
        }
        const int c = g.key[src];
        if (c < 0 || c >= g.ncells) {
            atomicOr(err, kErrGridIndex);
            continue;
        }
        const int s = g.off[c], e = g.off[c + 1];
        if (s < 0 || e > n || s > k || k >= e) {
            atomicOr(err, kErrGridIndex);
            continue;
        }
        if (e - s > kBigCell) continue;  // placed below, with its cell
        int r = 0;
        for (int j = s; j < e; ++j) r += g.perm[j].y < id;
        reorder_move(a, src, s + r, id, err);
    }
    const int nb = min(*g.nbig_snap, g.big_cap);
    for (int b = blockIdx.x; b < nb; b += gridDim.x) {
        const int c = g.big[b];
        if (c < 0 || c >= g.ncells) {
            if (threadIdx.x == 0) atomicOr(err, kErrGridIndex);
            continue;
        }
        const int s = g.off[c], e = g.off[c + 1];
        if (s < 0 || e > n || e - s <= kBigCell) {
            if (threadIdx.x == 0) atomicOr(err, kErrGridIndex);
            continue;
        }
        const int k = e - s;
        const int* sorted = block_sort_ids(g.perm + s, k, g.rank + s, g.sortbuf + s);
        __syncthreads();
        for (int j = threadIdx.x; j < k; j += blockDim.x) {
            const int2 pe = g.perm[s + j];
            const int src = pe.x, id = pe.y;
            if (src < 0 || src >= cap) {
                atomicOr(err, kErrGridIndex);
                continue;
            }
            reorder_move(a, src, s + lower_rank(sorted, k, id), id, err);
        }
        __syncthreads();  // the buffers are reused by the block's next cell
    }
}

size_t grid_bufs_bytes(int cap, int ncells, bool own_off) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    int ntiles = (ncells + kScanTile - 1) / kScanTile;
    if (ntiles < 1) ntiles = 1;
    const size_t big_cap = static_cast<size_t>(cap) / (kBigCell + 1) + 1;
    return al(sizeof(unsigned) * (size_t)ncells) + (own_off ? al(sizeof(int) * ((size_t)ncells + 1)) : 0) +
           al(sizeof(int) * (size_t)cap) * 3 + al(sizeof(int2) * (size_t)cap) + al(sizeof(unsigned) * (size_t)ntiles) +
           al(sizeof(int) * big_cap) + 256;
}

GridBufs grid_bufs_carve(void* base, int cap, int ncells, bool own_off) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    char* p = static_cast<char*>(base);
    GridBufs g;
    g.ncells = ncells;
    g.ntiles = (ncells + kScanTile - 1) / kScanTile;
    if (g.ntiles < 1) g.ntiles = 1;
    g.count = reinterpret_cast<unsigned*>(p);
    p += al(sizeof(unsigned) * (size_t)ncells);
    g.off = nullptr;
    if (own_off) {
        g.off = reinterpret_cast<int*>(p);
        p += al(sizeof(int) * ((size_t)ncells + 1));
    }
    g.key = reinterpret_cast<int*>(p);
    p += al(sizeof(int) * (size_t)cap);
    g.rank = reinterpret_cast<int*>(p);
    p += al(sizeof(int) * (size_t)cap);
    g.sortbuf = reinterpret_cast<int*>(p);
    p += al(sizeof(int) * (size_t)cap);
    g.perm = reinterpret_cast<int2*>(p);
    p += al(sizeof(int2) * (size_t)cap);
    g.tile_sum = reinterpret_cast<unsigned*>(p);
    p += al(sizeof(unsigned) * (size_t)g.ntiles);
    g.big_cap = cap / (kBigCell + 1) + 1;
    g.big = reinterpret_cast<int*>(p);
    p += al(sizeof(int) * static_cast<size_t>(g.big_cap));
    g.used = nullptr;
    g.total = reinterpret_cast<int*>(p);  // the last 256 bytes: total, nbig, nbig_snap
    g.nbig = g.total + 1;
    g.nbig_snap = g.total + 2;
    return g;
}

cudaError_t grid_keys_enqueue(const float2* pos, const int* n_ptr, int cap, float ox, float oy, float cell, int dimx,
                              int dimy, GridBufs g, cudaStream_t stream) {
    const int T = 256;
    k_grid_keys<<<particle_blocks(cap, T), T, 0, stream>>>(pos, n_ptr, ox, oy, cell, dimx, dimy, g.count, g.key,
                                                           g.rank, g.tile_sum);
    return cudaGetLastError();
}

cudaError_t grid_sort_enqueue(const int32_t* id, int* n_ptr, int cap, GridBufs g, ReorderArgs a,
                              unsigned* err, cudaStream_t stream) {
    const int T = 256;
    const int pb = particle_blocks(cap, T);
    const int sb = g.ntiles < 8 * sm_count() ? g.ntiles : 8 * sm_count();
    cudaError_t e;
    k_grid_scan<<<sb, kScanThreads, 0, stream>>>(g);
    if ((e = cudaMemsetAsync(g.tile_sum, 0, sizeof(unsigned) * g.ntiles, stream)) != cudaSuccess) return e;
    k_grid_scatter<<<pb, T, 0, stream>>>(n_ptr, id, g, err);
    k_grid_reorder<<<pb, kReorderThreads, 0, stream>>>(n_ptr, cap, g, a, err);
    return cudaGetLastError();
}

cudaError_t grid_build_enqueue(const float2* pos, const int32_t* id, int* n_ptr, int cap, float ox, float oy,
                               float cell, int dimx, int dimy, GridBufs g, ReorderArgs a, unsigned* err,
                               cudaStream_t stream) {
    cudaError_t e;
    if ((e = cudaMemsetAsync(g.count, 0, sizeof(unsigned) * static_cast<size_t>(g.ncells), stream)) != cudaSuccess)
        return e;
    if ((e = cudaMemsetAsync(g.tile_sum, 0, sizeof(unsigned) * g.ntiles, stream)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(g.nbig, 0, sizeof(int), stream)) != cudaSuccess) return e;
    if ((e = grid_keys_enqueue(pos, n_ptr, cap, ox, oy, cell, dimx, dimy, g, stream)) != cudaSuccess) return e;
    return grid_sort_enqueue(id, n_ptr, cap, g, a, err, stream);
}

__global__ void k_set_int(int* p, int v) { *p = v; }

}  // namespace tss

// ---------------------------------------------------------------------------
// C ABI: grid build on caller-owned device memory
// ---------------------------------------------------------------------------
namespace {
// workspace layout: [n + error word (256 B)] [grid buffers without the offset
// table, which is the caller's d_cell_off]
size_t ws_bytes(int n, int dimx, int dimy) {
    size_t cells = static_cast<size_t>(dimx) * static_cast<size_t>(dimy);
    int cap = n > 0 ? n : 1;
    return 256 + tss::grid_bufs_bytes(cap, static_cast<int>(cells), false);
}
}  // namespace

extern "C" tss_status tss_grid_workspace_size(int n, int dimx, int dimy, size_t* bytes) {
    if (!bytes || n < 0 || dimx <= 0 || dimy <= 0) return TSS_INVALID_ARG;
    if (static_cast<long long>(dimx) * dimy >= (1LL << 31) - 1) return TSS_INVALID_ARG;
    *bytes = ws_bytes(n, dimx, dimy);
    return TSS_OK;
}

extern "C" tss_status tss_grid_build(const float* d_pos, const int32_t* d_id, int n, float origin_x, float origin_y,
                                     float cell_size, int dimx, int dimy, int32_t* d_order, int32_t* d_cell_off,
                                     void* d_workspace, size_t workspace_bytes, void* stream) {
    if (n < 0 || dimx <= 0 || dimy <= 0 || !(cell_size > 0.0f) || !d_cell_off || !d_workspace) return TSS_INVALID_ARG;
    if (n > 0 && (!d_pos || !d_id || !d_order)) return TSS_INVALID_ARG;
    if (static_cast<long long>(dimx) * dimy >= (1LL << 31) - 1) return TSS_INVALID_ARG;
    if (workspace_bytes < ws_bytes(n, dimx, dimy)) return TSS_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int cells = dimx * dimy;
    const int cap = n > 0 ? n : 1;
    char* w = static_cast<char*>(d_workspace);
    int* n_dev = reinterpret_cast<int*>(w);
    unsigned* err = reinterpret_cast<unsigned*>(n_dev + 2);
    tss::GridBufs g = tss::grid_bufs_carve(w + 256, cap, cells, false);
    g.off = d_cell_off;  // write the offsets straight into the caller's table
    if (cudaMemsetAsync(w, 0, 256, st) != cudaSuccess) return TSS_CUDA_ERROR;
    tss::k_set_int<<<1, 1, 0, st>>>(n_dev, n);
    tss::ReorderArgs a{};  // only the order is gathered
    a.src_pos = reinterpret_cast<const float2*>(d_pos);
    a.dst_order = d_order;
    cudaError_t e = tss::grid_build_enqueue(reinterpret_cast<const float2*>(d_pos), d_id, n_dev, cap, origin_x, origin_y,
                                            cell_size, dimx, dimy, g, a, err, st);
    return e == cudaSuccess ? TSS_OK : TSS_CUDA_ERROR;
}
