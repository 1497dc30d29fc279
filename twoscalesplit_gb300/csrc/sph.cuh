// sph.cuh -- the gather kernels of one two-scale WCSPH step.
#pragma once
#include "grid.cuh"
#include "tss_device.cuh"

namespace tss {

// One scale's arrays.  "cur" arrays are in this step's (cell, id) order, "list"
// arrays (n*) hold the state the next step starts from, in that same order for
// existing particles, with newly created high-res children appended.
struct ScaleView {
    const float2* pos;
    const float2* vel;
    const uint8_t* st;
    const int32_t* id;
    float* dens;
    float* pres;
    float* q;        // p / rho^2
    float* tr;       // low scale: each split parent's tether radius, written by the low-res force
    // low scale, one byte per cell: the low-res force sets a cell to the step counter
    // (mod 256) when the cell holds an entry in state 0 after the split marks.  Any
    // other value only makes the high-res force walk a row it could skip.
    uint8_t* cflag;
    // Neighbour lists the density pass records for the force pass of the same scale
    // (one particle per thread): entry c of sorted particle i is
    // nbr[c * nbr_stride + i] = j - i for its c-th same-scale neighbour within the
    // density's support (itself left out), in window order; nnbr[i] is their count,
    // kNbrOverflow when there are more than kMaxNbr or an offset does not fit 16
    // bits.  Null when the density pass of this step did not record them.
    int16_t* nbr;
    uint8_t* nnbr;
    long long nbr_stride;  // entries per list column: the scale's capacity
    float2* acc;
    const int* off;  // dense cell offsets [C+1]
    int32_t* map;    // slot id -> index in the cur arrays
    float2* npos;
    float2* nvel;
    uint8_t* nst;
    int32_t* nid;
    float* ndens;    // carried densities/pressures (relaxation only; may be null)
    float* npres;
    // the next step's grid keys, written where the list entries are written
    unsigned* gcount;
    int* gkey;
    int* grank;
    unsigned* gtile;
};

struct StepView {
    ScaleView L, H;
    const float2* wpos;     // walls: each scene's in (low cell, id) order from its wall base
    const int* woff;        // wall cell offsets on the low grid
    const uint8_t* wnear;   // per low cell: 1 when a cell within two cells of it holds a wall particle
    Counters* cnt;
    uint8_t* split_flag;    // [n_low]
    int32_t* split_ids;     // [n_low] parents split this step (= next step's fresh list)
    unsigned* split_tile;   // [ceil(n_low / kSplitTile)] splits per tile, zero at step start
    float2* relax_pos;      // [capH] relaxation scratch
    float2* relax_vel;
    int nL;                 // low-res count (constant for a solver)
    // batches only: per-scene parameters and each sorted particle's scene
    const Params* table;
    const uint16_t* scL;
    const uint16_t* scH;
};

constexpr int kMaxNbr = 20;
constexpr uint8_t kNbrOverflow = 255;

constexpr int kSplitThreads = 256;
constexpr int kSplitItems = 16;
constexpr int kSplitTile = kSplitThreads * kSplitItems;

// B = false: one scene, parameters P0 (kernel constants).  B = true: a batch of
// scenes; each particle's parameters are V.table[scene of the particle], and each
// scene's grids sit at its cell bases in one global cell space.  The gathers
// (densities, forces) are further templated on how a particle's window is walked
// (gather.cuh) and launched through the launchers below.
template <bool B> __global__ void k_split(Params P0, StepView V);
template <bool B> __global__ void k_relax_density(Params P0, StepView V);
template <bool B> __global__ void k_relax_force(Params P0, StepView V);
__global__ void k_relax_apply(Params P0, StepView V);
__global__ void k_step_finish(Counters* c);

// host launchers (batched selects B; warp: one particle per warp instead of per
// thread; fast: FastArith instead of ExactArith, arith.cuh).  Gather g: 0 high-res
// density, 1 low-res density, 2 low-res force, 3 high-res force.
void launch_gather(int g, bool batched, bool warp, bool fast, int blocks, int threads, cudaStream_t s,
                   const Params& P, const StepView& V);
void launch_k_split(bool batched, int blocks, int threads, cudaStream_t s, const Params& P, const StepView& V);
void launch_k_relax_density(bool batched, int blocks, int threads, cudaStream_t s, const Params& P, const StepView& V);
void launch_k_relax_force(bool batched, int blocks, int threads, cudaStream_t s, const Params& P, const StepView& V);
// resident blocks per SM of gather g at `threads` threads per block; 0 on error
int gather_occupancy(int g, bool batched, bool warp, bool fast, int threads);
// wnear of one scene's dimx x dimy low grid from its wall cell offsets (both
// pointers at the scene's first cell), after its wall grid is built
void launch_wall_near(const int* woff, uint8_t* wnear, int dimx, int dimy, cudaStream_t s);

}  // namespace tss
