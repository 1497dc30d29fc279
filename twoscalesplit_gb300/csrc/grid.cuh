// grid.cuh -- uniform-grid neighbour structure on the GPU: a counting sort by cell
// with a per-cell fix-up into (cell, id) order.
//
// Replaces computeParticleHash + thrust::sort_by_key + memset +
// computeCellStartEndIndices (TwoScale2D/WCSPHSolver.cu:1246-1340, 2814-2854).
// The grids here have about as many cells as particles, so instead of a radix sort
// of cell keys the build counts particles per cell, scans the counts (that scan is
// also the dense cell-offset table the gathers need) and scatters; the order inside
// a cell is then fixed to ascending id, which makes the result independent of the
// atomic order and equal to a stable sort by cell of an id-ascending list.
//
//   k_grid_keys     key[i] = cell(pos[i]); rank[i] = atomicAdd(&count[cell], 1);
//                   per tile of kScanTile cells, the number of particles
//                   (warp-aggregated atomics), so the scan needs no look-back
//   k_grid_scan     off = exclusive_scan(count) over the cells in use: each tile
//                   adds the sums of the tiles before it; count is zeroed for the
//                   next build; off[used] = total = the number of keyed entries
//   k_grid_scatter  perm[off[key[i]] + rank[i]] = (i, id[i]); entries whose key is
//                   negative (removed since their key pass) are dropped
//   k_grid_reorder  each sorted slot finds its final place in its cell, ascending
//                   id, and gathers the particle's state there (SoA reorder); the
//                   list count becomes the sorted count.  In a cell of at most
//                   kBigCell entries the slot counts the smaller ids of its cell
//                   (k compares, the grids' cells hold a few particles); a larger
//                   cell -- particles clamped into a border cell, a collapsing flow,
//                   a caller's clustered points -- is taken whole by one block,
//                   which sorts its ids (LSD radix sort, 8-bit digits, O(k) per
//                   pass) and places each entry by a binary search, so no cell
//                   costs more than O(k log k)
#pragma once
#include "tss_device.cuh"

namespace tss {

// A scan tile of 2048 cells: the grids have about as many cells as particles, so
// the scan is latency-bound; 2048-cell tiles give the 1M-particle scene's 3.1M-cell
// high-res grid 1526 tiles (8 blocks per SM, one or two tiles each) and scanned it
// 6.7 us faster than 8192-cell tiles.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;
// Cells with more entries than this are ordered by a block-wide sort of their ids
// in the reorder (see above); at most total / (kBigCell + 1) cells can be that big.
constexpr int kBigCell = 32;
constexpr int kReorderThreads = 256;

struct GridBufs {
    int ncells;             // C
    unsigned* count;        // [C], zero between builds
    int* off;               // [C+1]
    int* key;               // [cap] cell of list entry i (negative: entry dropped at the next build)
    int* rank;              // [cap]
    int2* perm;             // [cap] (list index, id) in cell order (atomic order inside a cell)
    unsigned* tile_sum;     // [ntiles] particles per tile of kScanTile cells (zero between builds)
    int ntiles;
    const int* used;        // device int: cells [0, used) can hold entries (null: all C); the
                            // scan covers only those, so its cost follows the cells in use
    int* total;             // device int: entries sorted by the last build
    int* big;               // [big_cap] cells with more than kBigCell entries (the scan appends)
    int big_cap;            // cap / (kBigCell + 1) + 1
    int* nbig;              // device int: cells appended by the scan (the scatter resets it)
    int* nbig_snap;         // device int: ... as the scatter found it, for the reorder
    int* sortbuf;           // [cap] ids of the big cells while they are sorted (with rank)
};

// What the reorder moves: list-order arrays (src) into sorted-order arrays (dst).
struct ReorderArgs {
    const float2* src_pos;
    const float2* src_vel;     // may be null
    const uint8_t* src_st;     // may be null
    const float* src_dens;     // may be null (carried only for the relaxation)
    const float* src_pres;
    float2* dst_pos;
    float2* dst_vel;
    uint8_t* dst_st;
    int32_t* dst_id;
    float* dst_dens;
    float* dst_pres;
    int32_t* dst_order;        // may be null: source list index of each sorted position
    int32_t* slot_map;         // may be null: slot id -> sorted index
    int slots;                 // size of slot_map
    // batches: the scene of each sorted entry, page_scene[(id >> id_shift) >> page_shift]
    // (scenes own whole pages of low-res slots)
    uint16_t* dst_sc;          // may be null
    const uint16_t* page_scene;
    int page_shift;
    int id_shift;              // 0 for low-res ids, 2 for high-res (4 children per parent)
    int* h_state0;             // may be null: set to 1 if some entry has (state & 1) == 0
};

__global__ void k_grid_keys(const float2* __restrict__ pos, const int* __restrict__ n_ptr, float ox, float oy,
                            float cell, int dimx, int dimy, unsigned* __restrict__ count, int* __restrict__ key,
                            int* __restrict__ rank, unsigned* __restrict__ tile_sum);
__global__ void k_grid_scan(GridBufs g);
__global__ void k_grid_scatter(const int* __restrict__ n_ptr, const int32_t* __restrict__ id, GridBufs g,
                               unsigned* err);
__global__ void k_grid_reorder(int* n_ptr, int cap, GridBufs g, ReorderArgs a, unsigned* err);

// Enqueue a whole build: clears the counts and tile sums, then keys, scan,
// scatter, reorder.  `n_ptr` is a device int <= cap; inconsistent offsets set
// kErrGridIndex in *err.
cudaError_t grid_build_enqueue(const float2* pos, const int32_t* id, int* n_ptr, int cap, float ox, float oy,
                               float cell, int dimx, int dimy, GridBufs g, ReorderArgs a, unsigned* err,
                               cudaStream_t stream);
// The key pass alone (counts and tile sums must be zero), and the rest of a build
// (scan, clearing the tile sums for the next key pass, scatter, reorder).  The
// solver's step runs the key pass inside its force kernels (grid_key below) and
// only the rest here.
cudaError_t grid_keys_enqueue(const float2* pos, const int* n_ptr, int cap, float ox, float oy, float cell, int dimx,
                              int dimy, GridBufs g, cudaStream_t stream);
cudaError_t grid_sort_enqueue(const int32_t* id, int* n_ptr, int cap, GridBufs g, ReorderArgs a,
                              unsigned* err, cudaStream_t stream);

// The key of list entry i for the next build: its cell, its rank among the cell's
// entries (atomic order; the reorder fixes the order by id) and the tile sum.
// Lanes of a warp that hit the same tile add once.
__device__ __forceinline__ void grid_key(unsigned* __restrict__ count, int* __restrict__ key, int* __restrict__ rank,
                                         unsigned* __restrict__ tile_sum, int i, int c) {
    key[i] = c;
    rank[i] = static_cast<int>(atomicAdd(&count[c], 1u));
    const unsigned t = static_cast<unsigned>(c) / kScanTile;
    const unsigned peers = __match_any_sync(__activemask(), t);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&tile_sum[t], static_cast<unsigned>(__popc(peers)));
}

// Device bytes of a grid's buffers for `cap` entries and `ncells` cells; own_off =
// false leaves out the offset table (the caller then sets g.off to its own).
size_t grid_bufs_bytes(int cap, int ncells, bool own_off = true);
GridBufs grid_bufs_carve(void* base, int cap, int ncells, bool own_off = true);

int particle_blocks(int cap, int threads);
int sm_count();
__global__ void k_set_int(int* p, int v);

}  // namespace tss
