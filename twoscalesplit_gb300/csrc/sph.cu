// sph.cu -- the step's kernels other than the gathers (split compaction and
// children, relaxation, step finish), the gathers in the reference's arithmetic
// (gathers.cuh with ExactArith), and the launchers that pick the arithmetic.
#include "gathers.cuh"

namespace tss {

// ---------------------------------------------------------------------------
// Ordered stream compaction of the split flags (warp ballots + block scan; the
// tile's offset is the sum of the earlier tiles' counts that k_force_low left)
// and creation of the 4 children of each split (initSubParticlesAndAddToList,
// WCSPHSolver.cu:956-1005): children of the k-th split parent in sorted order
// take high-res list entries n_high + 4k + 0..3.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void make_children(const Params& P, const StepView& V, int i, int id, long long hb) {
    const float2 p = V.L.npos[i], v = V.L.nvel[i];
    const float rho = V.L.dens[i];
    // the current tree's offset (initSubParticlesAndAddToList, WCSPHSolver.cu:956-1005)
    // or the older snapshot's DIR_LEN * r (TwoScale2D-master/.../WCSPHSolver.cu:840-850)
    const float rad =
        P.older_place ? 0.35355339f * P.r
                      : static_cast<float>(0.5 * sqrt(static_cast<double>(P.mL) / (static_cast<double>(2.0f * rho) * kPi)));
    const float2 cp[4] = {make_float2(p.x + rad, p.y + rad), make_float2(p.x - rad, p.y + rad),
                          make_float2(p.x + rad, p.y - rad), make_float2(p.x - rad, p.y - rad)};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int h = static_cast<int>(hb) + c;
        V.H.npos[h] = cp[c];
        V.H.nvel[h] = v;
        V.H.nst[h] = 1;
        V.H.nid[h] = 4 * id + c;
        grid_key(V.H.gcount, V.H.gkey, V.H.grank, V.H.gtile, h,
                 P.cbH + cell_hash_s<1>(P, cp[c]));
        if (V.H.ndens) {
            V.H.ndens[h] = 0.0f;
            V.H.npres[h] = 0.0f;
        }
    }
}

template <bool B>
__global__ void __launch_bounds__(kSplitThreads) k_split(Params P0, StepView V) {
    __shared__ unsigned s_warp[kSplitThreads / 32];
    __shared__ unsigned s_red[kSplitThreads / 32];
    const int n = V.cnt->cur[0];
    const int nH = V.cnt->cur[1];
    // tiles of the list in use, strided over the blocks (a pool's list is sized for
    // its capacity); the last of them publishes the counts
    const int ntiles = n > 0 ? (n + kSplitTile - 1) / kSplitTile : 1;
    const int capH = P0.capH;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        // k_force_low counted this tile's flags: a tile without a split has nothing
        // to compact (only the last tile is always taken: it publishes the counts)
        if (tile != ntiles - 1 && V.split_tile[tile] == 0u) continue;
        unsigned before = 0;
        for (int t = threadIdx.x; t < tile; t += blockDim.x) before += V.split_tile[t];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
        if (lane == 0) s_red[warp] = before;
        // warp-striped items: item k of lane l of warp w is tile base + (w*K + k)*32 + l,
        // so each warp's ballots cover 32 consecutive particles in order
        const int wbase = tile * kSplitTile + warp * kSplitItems * 32;
        unsigned warp_count = 0;
        unsigned masks[kSplitItems];
#pragma unroll
        for (int k = 0; k < kSplitItems; ++k) {
            const int i = wbase + k * 32 + lane;
            const bool f = i < n && V.split_flag[i] != 0;
            masks[k] = __ballot_sync(0xffffffffu, f);
            warp_count += __popc(masks[k]);
        }
        if (lane == 0) s_warp[warp] = warp_count;
        __syncthreads();
        if (warp == 0) {
            unsigned w = lane < kSplitThreads / 32 ? s_warp[lane] : 0u;
            unsigned r = lane < kSplitThreads / 32 ? s_red[lane] : 0u;
            unsigned wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                unsigned t = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += t;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(0xffffffffu, r, o);
            if (lane < kSplitThreads / 32) s_warp[lane] = wi - w + r;
            const unsigned total = __shfl_sync(0xffffffffu, wi, kSplitThreads / 32 - 1) + r;
            if (lane == 0 && tile == ntiles - 1) {
                const int nsplit = static_cast<int>(total);
                long long want = static_cast<long long>(nH) + 4LL * nsplit;
                V.cnt->n_split = nsplit;
                if (want > capH) {
                    atomicOr(&V.cnt->err, kErrCapacity);
                    want = nH + 4LL * ((capH - nH) / 4);
                }
                V.cnt->next[1] = static_cast<int>(want);
                V.cnt->next[0] = n;
            }
        }
        __syncthreads();
        unsigned rank = s_warp[warp];
        const unsigned lt = (1u << lane) - 1u;
#pragma unroll
        for (int k = 0; k < kSplitItems; ++k) {
            const unsigned m = masks[k];
            if (m & (1u << lane)) {
                const int i = wbase + k * 32 + lane;
                const unsigned r = rank + __popc(m & lt);
                if (r < static_cast<unsigned>(n)) {
                    const int id = V.L.id[i];
                    V.split_ids[r] = id;
                    const long long hb = static_cast<long long>(nH) + 4LL * r;
                    if (hb + 4 <= capH) {
                        if constexpr (B) {
                            const Params& P = V.table[V.scL[i]];
                            make_children(P, V, i, id, hb);
                        } else {
                            make_children(P0, V, i, id, hb);
                        }
                    }
                }
            }
            rank += __popc(m);
        }
        __syncthreads();  // s_warp / s_red are reused by the next tile
    }
}

// ---------------------------------------------------------------------------
// Relaxation of the children created in the previous step (older snapshot,
// TwoScale2D-master/TwoScale2D/WCSPHSolver.cu:2380-2446): density 1133-1217,
// pressure + wall force 1499-1622 (= TwoScale2D/WCSPHSolver.cu:2035-2158), dt/10.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int fresh_child(const Params& P0, const StepView& V, int f) {
    const int slot = 4 * V.split_ids[f >> 2] + (f & 3);
    return (slot >= 0 && slot < P0.slotsH) ? V.H.map[slot] : -1;
}

__device__ __forceinline__ void relax_density_one(const Params& P, const StepView& V, int i) {
    const ScaleView& H = V.H;
    const ScaleView& L = V.L;
    const int* offH = H.off + P.cbH;
    const int* offL = L.off + P.cbL;
    const float2 p = H.pos[i];
    float d = 0.0f, dl = 0.0f;
    int csx, csy, cex, cey;
    grid_coord_s<1>(P, p.x, p.y, -P.rh, csx, csy);
    grid_coord_s<1>(P, p.x, p.y, P.rh, cex, cey);
    for (int cy = csy; cy <= cey; ++cy) {
        const int row = cy * P.dimH[0];
        const int b = offH[row + cex + 1];
        for (int j = offH[row + csx]; j < b; ++j) {
            float dist = vnorm(sub(p, H.pos[j]));
            if (dist <= P.rh) d += kernW(dist, P.rh, P.CH);
        }
    }
    grid_coord_s<0>(P, p.x, p.y, -P.rh, csx, csy);
    grid_coord_s<0>(P, p.x, p.y, P.rh, cex, cey);
    for (int cy = csy; cy <= cey; ++cy) {
        const int row = cy * P.dimL[0];
        const int b = offL[row + cex + 1];
        for (int j = offL[row + csx]; j < b; ++j) {
            float dist = vnorm(sub(p, L.pos[j]));
            if (dist <= P.rh) dl += kernW(dist, P.rh, P.CH);
        }
    }
    d *= P.mH;
    dl *= P.mL;
    d += dl;
    H.dens[i] = d;
    H.pres[i] = tait(d, P);
}

template <bool B>
__global__ void __launch_bounds__(256) k_relax_density(Params P0, StepView V) {
    const int nf = min(4 * V.cnt->n_fresh, P0.capH);  // relaxation scratch holds capH entries
    for (int f = tid(); f < nf; f += nthreads()) {
        const int i = fresh_child(P0, V, f);
        if (i < 0) continue;
        if constexpr (B) {
            const Params& P = V.table[V.scH[i]];
            relax_density_one(P, V, i);
        } else {
            relax_density_one(P0, V, i);
        }
    }
}

__device__ __forceinline__ void relax_force_one(const Params& P, const StepView& V, int i, int f) {
    const ScaleView& H = V.H;
    const ScaleView& L = V.L;
    const int* offH = H.off + P.cbH;
    const int* offL = L.off + P.cbL;
    const int* woff = V.woff + P.cbL;
    const float2* wpos = V.wpos + P.wb;
    float2 p = H.pos[i], v = H.vel[i];
    const float dens = H.dens[i], pre = H.pres[i];
    const float dens2 = dens * dens;
    float2 acc = make_float2(0.f, 0.f), accL = make_float2(0.f, 0.f), accB = make_float2(0.f, 0.f);
    int csx, csy, cex, cey;
    grid_coord_s<1>(P, p.x, p.y, -P.rh, csx, csy);
    grid_coord_s<1>(P, p.x, p.y, P.rh, cex, cey);
    for (int cy = csy; cy <= cey; ++cy) {
        const int row = cy * P.dimH[0];
        const int b = offH[row + cex + 1];
        for (int j = offH[row + csx]; j < b; ++j) {
            const float2 pij = sub(p, H.pos[j]);
            const float dist = vnorm(pij);
            if (dist != 0.0f && dist < P.rh) {
                const float dj = H.dens[j];
                const float coeff = pre / dens2 + H.pres[j] / (dj * dj);
                const float2 g = kernDW(pij, dist, P.rh, P.GH);
                acc.x += coeff * g.x;
                acc.y += coeff * g.y;
            }
        }
    }
    grid_coord_s<0>(P, p.x, p.y, -P.rh, csx, csy);
    grid_coord_s<0>(P, p.x, p.y, P.rh, cex, cey);
    for (int cy = csy; cy <= cey; ++cy) {
        const int row = cy * P.dimL[0];
        const int b = offL[row + cex + 1];
        for (int j = offL[row + csx]; j < b; ++j) {
            const float2 pij = sub(p, L.pos[j]);
            const float dist = vnorm(pij);
            if (dist != 0.0f && dist < P.rh) {
                const float dj = L.dens[j];
                const float coeff = pre / dens2 + L.pres[j] / (dj * dj);
                const float2 g = kernDW(pij, dist, P.rh, P.GH);
                accL.x += coeff * g.x;
                accL.y += coeff * g.y;
            }
        }
        const int wb = woff[row + cex + 1];
        for (int k = woff[row + csx]; k < wb; ++k) {
            const float2 pik = sub(p, wpos[k]);
            const float gm = wall_weight(vnorm(pik), P.rh, P.cs);
            accB.x += P.cBH * gm * pik.x;
            accB.y += P.cBH * gm * pik.y;
        }
    }
    acc.x *= -P.mH;
    acc.y *= -P.mH;
    accL.x *= -P.mL;
    accL.y *= -P.mL;
    acc.x += accL.x;
    acc.y += accL.y;
    acc.x += accB.x;
    acc.y += accB.y;
    v.x += P.relax_dt * acc.x;
    v.y += P.relax_dt * acc.y;
    p.x += P.relax_dt * v.x;
    p.y += P.relax_dt * v.y;
    V.relax_pos[f] = p;
    V.relax_vel[f] = v;
}

template <bool B>
__global__ void __launch_bounds__(256) k_relax_force(Params P0, StepView V) {
    const int nf = min(4 * V.cnt->n_fresh, P0.capH);  // relaxation scratch holds capH entries
    for (int f = tid(); f < nf; f += nthreads()) {
        const int i = fresh_child(P0, V, f);
        if (i < 0) continue;
        if constexpr (B) {
            const Params& P = V.table[V.scH[i]];
            relax_force_one(P, V, i, f);
        } else {
            relax_force_one(P0, V, i, f);
        }
    }
}

__global__ void k_relax_apply(Params P0, StepView V) {
    const int nf = min(4 * V.cnt->n_fresh, P0.capH);  // relaxation scratch holds capH entries
    for (int f = tid(); f < nf; f += nthreads()) {
        const int i = fresh_child(P0, V, f);
        if (i < 0) continue;
        const_cast<float2*>(V.H.pos)[i] = V.relax_pos[f];
        const_cast<float2*>(V.H.vel)[i] = V.relax_vel[f];
    }
}

__global__ void k_step_finish(Counters* c) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        c->sorted[0] = c->cur[0];
        c->sorted[1] = c->cur[1];
        c->cur[0] = c->next[0];
        c->cur[1] = c->next[1];
        c->n_fresh = c->n_split;
        c->h_state0 = 0;
        c->steps += 1;
        c->dropped = c->n_drop;
        c->total_split += c->n_split;
        c->total_removed += c->n_drop;
        c->n_drop = 0;
    }
}

// Host-side launchers.  The gathers come in two arithmetics: ExactArith here,
// FastArith in sph_fast.cu (launch_gather_fast, gather_occupancy_fast).
void launch_gather_fast(int g, bool batched, bool warp, int blocks, int threads, cudaStream_t s, const Params& P,
                        const StepView& V);
int gather_occupancy_fast(int g, bool batched, bool warp, int threads);

void launch_gather(int g, bool batched, bool warp, bool fast, int blocks, int threads, cudaStream_t s,
                   const Params& P, const StepView& V) {
    if (fast)
        launch_gather_fast(g, batched, warp, blocks, threads, s, P, V);
    else
        launch_gather_a<ExactArith>(g, batched, warp, blocks, threads, s, P, V);
}

int gather_occupancy(int g, bool batched, bool warp, bool fast, int threads) {
    return fast ? gather_occupancy_fast(g, batched, warp, threads)
                : gather_occupancy_a<ExactArith>(g, batched, warp, threads);
}

// Walls do not move: once per scene, each low cell records whether a wall particle
// lies in a cell within two cells of it (Chebyshev distance, inside the grid).
__global__ void k_wall_near(const int* __restrict__ woff, uint8_t* __restrict__ wnear, int dimx, int dimy) {
    const long long n = static_cast<long long>(dimx) * dimy;
    for (long long c = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; c < n;
         c += static_cast<long long>(gridDim.x) * blockDim.x) {
        const int cx = static_cast<int>(c % dimx), cy = static_cast<int>(c / dimx);
        const int x0 = max(cx - 2, 0), x1 = min(cx + 2, dimx - 1);
        bool any = false;
        for (int y = max(cy - 2, 0); y <= min(cy + 2, dimy - 1); ++y) {
            const long long row = static_cast<long long>(y) * dimx;
            any |= woff[row + x0] != woff[row + x1 + 1];
        }
        wnear[c] = any ? 1 : 0;
    }
}

void launch_wall_near(const int* woff, uint8_t* wnear, int dimx, int dimy, cudaStream_t s) {
    const long long n = static_cast<long long>(dimx) * dimy;
    if (n <= 0) return;
    const long long want = (n + 255) / 256;
    const int blocks = static_cast<int>(want < 16LL * sm_count() ? want : 16LL * sm_count());
    k_wall_near<<<blocks, 256, 0, s>>>(woff, wnear, dimx, dimy);
}

#define TSS_LAUNCHER(NAME)                                                                        \
    void launch_##NAME(bool batched, int blocks, int threads, cudaStream_t s, const Params& P,   \
                       const StepView& V) {                                                       \
        if (batched)                                                                              \
            NAME<true><<<blocks, threads, 0, s>>>(P, V);                                          \
        else                                                                                      \
            NAME<false><<<blocks, threads, 0, s>>>(P, V);                                         \
    }
TSS_LAUNCHER(k_split)
TSS_LAUNCHER(k_relax_density)
TSS_LAUNCHER(k_relax_force)
#undef TSS_LAUNCHER

}  // namespace tss
