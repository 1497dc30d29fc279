// gathers.cuh -- the four gather kernels of the two-scale step (densities of both
// scales, low-res force + advance + split marks, high-res force + integrate +
// tether), templated on the batch form B, the walk G (gather.cuh) and the
// arithmetic policy A (arith.cuh).  sph.cu instantiates them with ExactArith (the
// reference's bits), sph_fast.cu with FastArith (within the step's tolerance).
//
// Particles are in (cell, id) order.  Because the arrays are sorted by cell, the
// candidates of one row of the 3x3 (or wider cross-scale) cell window are one
// contiguous span [off[row + cx0], off[row + cx1 + 1]).  Each particle's sums take
// its candidates in the reference's order (cells row by row, particles in cell
// order), which keeps every FP32 sum identical to the reference's for the same
// list order.  The gathers walk a particle's window one of two ways (gather.cuh):
// one particle per thread, consecutive threads walking overlapping spans so that
// neighbour loads are shared through L1 (the throughput form), or one particle per
// warp with the candidates spread over the lanes (for scenes too small to fill the
// GPU); both give the same bits.
//
// Each kernel's per-particle work is an inlined function of the particle's Params:
// the kernel's own constants for a single scene, the scene's table row for a
// batch.  The row is read through a reference, so each field is loaded where it is
// used: a copy of the whole row kept every field live in registers across the
// neighbour loops, and the batched gathers spilled and ran 5 % slower.  A scene's
// cell windows index its grid at its cell base in the global cell space, so one
// sort and one offset table serve all scenes of a batch.
#pragma once
#include "arith.cuh"
#include "gather.cuh"
#include "sph.cuh"

namespace tss {

namespace gather_detail {
__device__ __forceinline__ int nthreads() { return gridDim.x * blockDim.x; }
__device__ __forceinline__ int tid() { return blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return sub2(a, b); }
__device__ __forceinline__ void add_density(float& d, float t) { d += t; }

// The particles of a gather, one per thread (G = PerThread) or one per warp
// (G = PerWarp, every lane of the warp taking the same particle).
template <class G, class F>
__device__ __forceinline__ void for_each_particle(int n, F&& f) {
    if constexpr (G::kWarp) {
        const int nw = nthreads() >> 5;
        for (int i = tid() >> 5; i < n; i += nw) f(i);
    } else {
        for (int i = tid(); i < n; i += nthreads()) f(i);
    }
}
}  // namespace gather_detail
using namespace gather_detail;

// Neighbour lists (ScaleView::nbr).  A density pass that runs one particle per
// thread records the same-scale candidates its window accepts, in window order,
// and the force pass of the same step walks that list instead of its window: the
// force's own candidates are a subset of the density's (same positions and
// states, cutoff d < r and d != 0 against d <= r, the same lambda masks), so
// testing each listed candidate again with the force's test gives the force's
// candidates in the same order -- the same sums, bit for bit -- without scanning
// the ~36 candidates of the window, of which about a third are accepted.  A
// particle with more than kMaxNbr neighbours, or one whose offset does not fit
// 16 bits, is marked and walks its window.
//
// The entries are staged in shared memory as they are found (`col`: the thread's
// column of a kMaxNbr x kNbrCols array, stride kNbrCols) and written out after the
// walk, entry c of every lane together, so that a warp's stores to the transposed
// global array coalesce; stored as found, they scattered over its rows.
constexpr int kNbrCols = 256;  // the gathers' largest block

struct NbrRecord {
    int16_t* col;
    int i, n;
    bool ok;
    __device__ __forceinline__ NbrRecord(int i_, int16_t* col_) : col(col_), i(i_), n(0), ok(true) {}
    __device__ __forceinline__ void add(int j) {
        if (j == i) return;  // the density's self term: never a force pair
        const int dj = j - i;
        if (n < kMaxNbr && dj >= -32768 && dj <= 32767) col[n * kNbrCols] = static_cast<int16_t>(dj);
        else ok = false;
        ++n;
    }
    __device__ __forceinline__ void finish(const ScaleView& S) const {
        if (ok) {
            int16_t* dst = S.nbr + i;  // 64-bit steps: a pool's capacity times kMaxNbr passes 2^31
            for (int c = 0; c < n; ++c, dst += S.nbr_stride) *dst = col[c * kNbrCols];
        }
        S.nnbr[i] = ok ? static_cast<uint8_t>(n) : kNbrOverflow;
    }
};

// A same-scale neighbour's state as the force pass reads it.
struct NbrState {
    float2 pos, vel;
    float q, dens;
    unsigned st;
};
__device__ __forceinline__ NbrState fetch_nbr(const ScaleView& S, int k) {
    return NbrState{S.pos[k], S.vel[k], S.q[k], S.dens[k], S.st[k]};
}

// Entries of a neighbour list taken per trip of the force pass's list walk (1 or 2).
constexpr int kListPairsPerTrip = 2;

// The force pass's same-scale pairs: from the list when there is one (test and
// term take the neighbour's NbrState), else `walk`.  Two entries per trip: both
// neighbours' state is loaded before either pair is evaluated, in list order, so
// that a thread has two neighbours' loads in flight (the force kernels wait mostly
// on these loads).  On a developed 1M-particle dam break that took k_force_high
// from 0.149 to 0.133 ms (exact) and 0.110 to 0.094 ms (tolerance arithmetic)
// against one per trip; four per trip was 3-8 % slower than two, with or without
// one block per SM fewer for the registers.
template <class G, class T, class Test, class Term, class Add, class Walk>
__device__ __forceinline__ void list_or_walk(const ScaleView& S, int i, Test&& test, Term&& term, Add&& add,
                                             T& sum, Walk&& walk) {
    if constexpr (!G::kWarp) {
        const int nc = S.nbr ? S.nnbr[i] : kNbrOverflow;
        if (nc != kNbrOverflow) {
            const long long stride = S.nbr_stride;
            const int16_t* src = S.nbr + i;
            int c = 0;
            if constexpr (kListPairsPerTrip == 2) {
                for (; c + 1 < nc; c += 2, src += 2 * stride) {
                    const int k0 = i + src[0], k1 = i + src[stride];
                    const NbrState n0 = fetch_nbr(S, k0), n1 = fetch_nbr(S, k1);
                    if (test(n0)) add(sum, term(n0));
                    if (test(n1)) add(sum, term(n1));
                }
            }
            for (; c < nc; ++c, src += stride) {
                const NbrState n0 = fetch_nbr(S, i + *src);
                if (test(n0)) add(sum, term(n0));
            }
            return;
        }
    }
    walk();
}

// ---------------------------------------------------------------------------
// High-res density + Tait, computeParticleDensityPressureHigh (WCSPHSolver.cu:1426-1516)
// ---------------------------------------------------------------------------
template <class A, class G>
__device__ __forceinline__ void density_high_one(const Params& P, const StepView& V, int i, bool hstate0,
                                                 int16_t* nbr_col) {
    const ScaleView& H = V.H;
    const ScaleView& L = V.L;
    const int* offH = H.off + P.cbH;
    const int* offL = L.off + P.cbL;
    const float2 p = H.pos[i];
    const unsigned s = H.st[i];
    float d = 0.0f, dl = 0.0f;
    float x = 0.0f;
    const auto term = [&](int) { return A::density(P, x); };
    const bool rec_on = !G::kWarp && H.nbr != nullptr;
    NbrRecord rec(i, nbr_col);
    int csx, csy, cex, cey;
    grid_coord_s<1>(P, p.x, p.y, -P.rh, csx, csy);
    grid_coord_s<1>(P, p.x, p.y, P.rh, cex, cey);
    // a candidate the lambda mask rejects gets key +inf: no cutoff passes it
    G::template window_keyed<4>(
        offH, P.dimH[0], csx, cex, csy, cey,
        [&](int k) { return lamHH(s, H.st[k]) ? sq(sub(p, H.pos[k])) : INFINITY; },
        [&](float xk) { return xk <= P.Tle_rh; },
        [&](int j, float xj) {
            if (rec_on) rec.add(j);
            return A::density(P, xj);
        },
        add_density, d);
    if (rec_on) rec.finish(H);
    grid_coord_s<0>(P, p.x, p.y, -P.r, csx, csy);
    grid_coord_s<0>(P, p.x, p.y, P.r, cex, cey);
    // With no high-res entry in state 0 in this step (hstate0 false), a state-1
    // particle's Q1 term can take only never-created slots (position (0,0), state 0:
    // lambda_HL rejects every existing state-1 entry), and those only when the
    // particle lies within r_h of (0,0): otherwise the walk adds nothing and is
    // skipped -- the same terms, none.
    const bool q1_live = hstate0 || (s & 1u) == 0u || sq(p) <= P.Tle_rh;
    if (P.q1 && q1_live) {
        // The reference reads the HIGH sorted list at LOW-grid ranges of its own
        // scene; past the scene's n_high that list still holds its initial identity
        // (slot t at position t).  A row's range [a, b) of low-list positions t
        // (t - baseL >= 0: offsets only grow) is taken in two runs, in order: the
        // positions below baseL + n_high, which are the high-list entries
        // t - baseL + baseH, and the rest, through the slot map.
        const int baseL = offL[0], baseH = offH[0];
        const int nHs = offH[P.CHs] - baseH;
        const int tH = baseL + nHs;   // first position past the scene's high-res list
        const int dH = baseH - baseL;  // low-list position -> high-list entry
        for (int cy = csy; cy <= cey; ++cy) {
            const int row = cy * P.dimL[0];
            const int a = offL[row + csx], b = offL[row + cex + 1];
            const int m = min(b, max(a, tH));
            G::span(
                a + dH, m + dH,
                [&](int k) {
                    if (!lamHL(s, H.st[k])) return false;
                    x = sq(sub(p, H.pos[k]));
                    return x <= P.Tle_rh;
                },
                term, add_density, d);
            G::span(
                m, b,
                [&](int t) {
                    const int tl = t - baseL;
                    const int slot = 4 * P.sbL + tl;
                    const int k = (tl < 4 * P.nLs && slot < P.slotsH) ? H.map[slot] : -1;
                    float2 pj = make_float2(0.0f, 0.0f);
                    unsigned sj = 0;
                    if (k >= 0) {
                        pj = H.pos[k];
                        sj = H.st[k];
                    }
                    if (!lamHL(s, sj)) return false;
                    x = sq(sub(p, pj));
                    return x <= P.Tle_rh;
                },
                term, add_density, d);
        }
    } else if (!P.q1) {
        G::window(
            offL, P.dimL[0], csx, cex, csy, cey,
            [&](int k) {
                if (!lamHL(s, L.st[k])) return false;
                x = sq(sub(p, L.pos[k]));
                return x <= P.Tle_rh;
            },
            term, add_density, dl);
    }
    d *= P.mH;
    dl *= P.mL;
    d += dl;
    const float pr = tait(d, P);
    if (G::leader()) {
        H.dens[i] = d;
        H.pres[i] = pr;
        H.q[i] = pr / (d * d);
        if (!isfinite(d) || !isfinite(pr)) atomicOr(&V.cnt->err, kErrNumeric);
    }
}

template <bool B, class G, class A>
__global__ void __launch_bounds__(256) k_density_high(Params P0, StepView V) {
    __shared__ int16_t s_nbr[G::kWarp ? 1 : kMaxNbr * kNbrCols];
    int16_t* const nbr_col = s_nbr + (G::kWarp ? 0 : threadIdx.x);
    const bool hstate0 = V.cnt->h_state0 != 0;
    for_each_particle<G>(V.cnt->cur[1], [&](int i) {
        if constexpr (B) {
            const Params& P = V.table[V.scH[i]];
            density_high_one<A, G>(P, V, i, hstate0, nbr_col);
        } else {
            density_high_one<A, G>(P0, V, i, hstate0, nbr_col);
        }
    });
}

// ---------------------------------------------------------------------------
// Low-res density + Tait, computeParticleDensityPressure (WCSPHSolver.cu:1342-1424)
// ---------------------------------------------------------------------------
template <class A, class G>
__device__ __forceinline__ void density_low_one(const Params& P, const StepView& V, int i, bool cross,
                                                int16_t* nbr_col) {
    const ScaleView& H = V.H;
    const ScaleView& L = V.L;
    const float2 p = L.pos[i];
    const unsigned s = L.st[i];
    float d = 0.0f, dh = 0.0f;
    float x = 0.0f;
    const auto term = [&](int) { return A::density(P, x); };
    const bool rec_on = !G::kWarp && L.nbr != nullptr;
    NbrRecord rec(i, nbr_col);
    int csx, csy, cex, cey;
    grid_coord_s<0>(P, p.x, p.y, -P.r, csx, csy);
    grid_coord_s<0>(P, p.x, p.y, P.r, cex, cey);
    G::template window_keyed<2>(
        L.off + P.cbL, P.dimL[0], csx, cex, csy, cey, [&](int k) { return sq(sub(p, L.pos[k])); },
        [&](float xk) { return xk <= P.Tle_r; },
        [&](int j, float xj) {
            if (rec_on) rec.add(j);
            return A::density(P, xj);
        },
        add_density, d);
    if (rec_on) rec.finish(L);
    if (cross) {  // only state-0 high-res particles can contribute (lambda_LH)
        grid_coord_s<1>(P, p.x, p.y, -P.r, csx, csy);
        grid_coord_s<1>(P, p.x, p.y, P.r, cex, cey);
        G::window(
            H.off + P.cbH, P.dimH[0], csx, cex, csy, cey,
            [&](int k) {
                if (!lamLH(s, H.st[k])) return false;
                x = sq(sub(p, H.pos[k]));
                return x <= P.Tle_r;
            },
            term, add_density, dh);
    }
    d *= P.mL;
    dh *= P.mH;
    const float rho = d + dh;
    const float pr = tait(rho, P);
    if (G::leader()) {
        L.dens[i] = rho;
        L.pres[i] = pr;
        L.q[i] = pr / (rho * rho);
        if (!isfinite(rho) || !isfinite(pr)) atomicOr(&V.cnt->err, kErrNumeric);
    }
}

template <bool B, class G, class A>
__global__ void __launch_bounds__(256) k_density_low(Params P0, StepView V) {
    __shared__ int16_t s_nbr[G::kWarp ? 1 : kMaxNbr * kNbrCols];
    int16_t* const nbr_col = s_nbr + (G::kWarp ? 0 : threadIdx.x);
    const bool cross = V.cnt->h_state0 != 0;
    for_each_particle<G>(V.cnt->cur[0], [&](int i) {
        if constexpr (B) {
            const Params& P = V.table[V.scL[i]];
            density_low_one<A, G>(P, V, i, cross, nbr_col);
        } else {
            density_low_one<A, G>(P0, V, i, cross, nbr_col);
        }
    });
}

// Wall term of a force sum (updateAccCell 562-579 / updateAccCellComplementHigh
// 867-884): every wall particle of the window's cells, in cell order.  Pairs with
// sqrtf(x) > rad have q >= 2 and add exactly zero, so they are skipped.  S selects
// the scale: 0 the low-res radius r, 1 the high-res radius rh.
template <class A, class G, int S>
__device__ __forceinline__ float2 wall_sum(const Params& P, const StepView& V, float2 p, int csx, int cex, int csy,
                                           int cey, float Tle, float cB) {
    float2 accB = make_float2(0.f, 0.f);
    // A window of at most four cells a side from (csx, csy) lies within two cells of
    // (mx, my); with no wall particle there the sum is empty.
    if (cex - csx <= 3 && cey - csy <= 3) {
        const int mx = min(csx + 1, P.dimL[0] - 1), my = min(csy + 1, P.dimL[1] - 1);
        if (!V.wnear[P.cbL + my * P.dimL[0] + mx]) return accB;
    }
    const int* woff = V.woff + P.cbL;
    const float2* wpos = V.wpos + P.wb;
    float2 pik = make_float2(0.f, 0.f);
    float x = 0.0f;
    for (int cy = csy; cy <= cey; ++cy) {
        const int row = cy * P.dimL[0];
        G::span(
            woff[row + csx], woff[row + cex + 1],
            [&](int k) {
                pik = sub(p, wpos[k]);
                x = sq(pik);
                return !(x > Tle);  // NaN passes: the reference's 0 * NaN offset propagates it
            },
            [&](int) { return A::template wall<S>(P, pik, x, cB); },
            [](float2& a, float2 t) {
                a.x += t.x;
                a.y += t.y;
            },
            accB);
    }
    return accB;
}

// ---------------------------------------------------------------------------
// Low-res force + advance + split test: computeParticleAcceleration
// (WCSPHSolver.cu:1648-1865) with advance (1604-1646) fused; its predicted position
// is the advanced position bit for bit.  The fluid and wall sums are independent
// accumulators, so they are taken in two passes over the window.  The new position
// also gives the entry's key for the next step's grid.  Returns the split flag.
// ---------------------------------------------------------------------------
template <class A, class G>
__device__ __forceinline__ bool force_low_one(const Params& P, const StepView& V, int i, bool cross) {
    const ScaleView& H = V.H;
    const ScaleView& L = V.L;
    float2 p = L.pos[i], v = L.vel[i];
    const unsigned s = L.st[i];
    const float dens = L.dens[i], qi = L.q[i];
    PairTerms fl{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};  // (acc, accT)
    float2 pij = make_float2(0.f, 0.f);
    float x = 0.0f;
    int csx, csy, cex, cey;
    grid_coord_s<0>(P, p.x, p.y, -P.r, csx, csy);
    grid_coord_s<0>(P, p.x, p.y, P.r, cex, cey);
    {
        const auto test = [&](int k) {
            pij = sub(p, L.pos[k]);
            x = sq(pij);
            return x != 0.0f && x <= P.Tlt_r && notDeleted(L.st[k]);
        };
        const auto term = [&](int j) {
            return A::template pair<kHLow>(P, pij, x, sub(v, L.vel[j]), qi, L.q[j], dens, L.dens[j]);
        };
        const auto test_n = [&](const NbrState& n) {
            pij = sub(p, n.pos);
            x = sq(pij);
            return x != 0.0f && x <= P.Tlt_r && notDeleted(n.st);
        };
        const auto term_n = [&](const NbrState& n) {
            return A::template pair<kHLow>(P, pij, x, sub(v, n.vel), qi, n.q, dens, n.dens);
        };
        list_or_walk<G>(L, i, test_n, term_n, add_terms, fl,
                        [&] { G::window(L.off + P.cbL, P.dimL[0], csx, cex, csy, cey, test, term, add_terms, fl); });
    }
    const float2 accB = wall_sum<A, G, 0>(P, V, p, csx, cex, csy, cey, P.Tle_r, P.cBL);
    PairTerms fh{make_float2(0.f, 0.f), fl.t};  // (accH, accT): the sigma sum continues
    if (cross) {
        grid_coord_s<1>(P, p.x, p.y, -P.r, csx, csy);
        grid_coord_s<1>(P, p.x, p.y, P.r, cex, cey);
        G::window(
            H.off + P.cbH, P.dimH[0], csx, cex, csy, cey,
            [&](int k) {
                if (!lamLH(s, H.st[k])) return false;
                pij = sub(p, H.pos[k]);
                x = sq(pij);
                return x != 0.0f && x <= P.Tlt_r;
            },
            [&](int j) {
                return A::template pair<kHCross>(P, pij, x, sub(v, H.vel[j]), qi, H.q[j], dens, H.dens[j]);
            },
            add_terms, fh);
    }
    float2 acc = fl.a, accH = fh.a;
    const float2 accT = fh.t;
    acc.x *= -P.mL;
    acc.y *= -P.mL;
    accH.x *= -P.mH;
    accH.y *= -P.mH;
    acc.x += accH.x;
    acc.y += accH.y;
    acc.x -= P.sigma * accT.x;
    acc.y -= P.sigma * accT.y;
    acc.x += accB.x;
    acc.y += accB.y;
    acc.y -= P.g;
    v.x += P.dt * acc.x;
    v.y += P.dt * acc.y;
    p.x += P.dt * v.x;
    p.y += P.dt * v.y;
    // split test on the predicted position (computeParticleAcceleration 1810-1835)
    // against the ROI of this step; with TSS_FLAG_MERGE a split parent outside it
    // merges back
    const float kf = static_cast<float>(V.cnt->steps - P.step0);
    const float rx0 = P.roi[0] + kf * P.roi_vdt[0], rx1 = P.roi[2] + kf * P.roi_vdt[0];
    const float ry0 = P.roi[1] + kf * P.roi_vdt[1], ry1 = P.roi[3] + kf * P.roi_vdt[1];
    const bool in_roi = rx0 < p.x && p.x < rx1 && ry0 < p.y && p.y < ry1;
    bool flag = false;
    uint8_t ns = static_cast<uint8_t>(s);
    if (s == 0u && in_roi) {
        ns = 1;
        flag = true;
    } else if (P.merge && s == 1u && !in_roi) {
        ns = 0;
    }
    if (G::leader()) {
        L.acc[i] = acc;
        if (!isfinite(acc.x) || !isfinite(acc.y)) atomicOr(&V.cnt->err, kErrNumeric);
        // a split parent's tether radius, 0.75 sqrt(m / (rho pi)) in double as the
        // reference evaluates it (adjustPosition, WCSPHSolver.cu:1007-1022), once per
        // parent here instead of once per child in the high-res force: FP64 is slow
        // on this GPU.  min(dist, float(R)) == float(min(dist, R)) for a float dist
        // (rounding is monotone), so the children's clamp is unchanged bit for bit.
        if (s == 1u)
            L.tr[i] = static_cast<float>(0.75 * sqrt(static_cast<double>(P.mL) / (static_cast<double>(dens) * kPi)));
        // the cells of this step's grid that hold an entry in state 0 after the split
        // marks: the only low-res partners of a state-1 child in the high-res force.
        // The entry's cell is the one its key was made from (its position at the
        // start of the step, the same cell function).
        if (ns == 0u) L.cflag[P.cbL + cell_hash_s<0>(P, L.pos[i])] = static_cast<uint8_t>(V.cnt->steps);
        L.npos[i] = p;
        L.nvel[i] = v;
        L.nid[i] = L.id[i];
        grid_key(L.gcount, L.gkey, L.grank, L.gtile, i,
                 P.cbL + cell_hash_s<0>(P, p));
        L.nst[i] = ns;
        V.split_flag[i] = flag ? 1 : 0;
        if (L.ndens) {
            L.ndens[i] = dens;
            L.npres[i] = L.pres[i];
        }
    }
    return flag;
}

// One particle per thread: a warp-uniform loop (every lane makes the same number of
// trips, lanes past n inactive) so the ballot that feeds the split compaction sees
// whole warps; a warp's 32 particles lie in one compaction tile (kSplitTile % 32 ==
// 0).  One particle per warp: the leader counts its particle's split.
// 48 registers (five blocks per SM) in both forms of the exact arithmetic.  The
// batched form measured the same at 40 and 48 on a batch of 512 mixed scenes (4.11
// / 4.08 ms), 3-7 % faster at 48 on batches of one scene, and 10 % slower at 64.
// The single-scene form in the tolerance arithmetic fits 40 registers without
// spilling and runs six blocks per SM: 3.5 % faster on the developed 1M dam break
// (0.130 -> 0.125 ms); batched, it would spill 76 bytes at 40 and keeps 48.
template <bool B, class G, class A>
__global__ void __launch_bounds__(256, (A::kFast && !B) ? 6 : 5) k_force_low(Params P0, StepView V) {
    const int n = V.cnt->cur[0];
    const bool cross = V.cnt->h_state0 != 0;
    const auto one = [&](int i) {
        if constexpr (B) {
            const Params& P = V.table[V.scL[i]];
            return force_low_one<A, G>(P, V, i, cross);
        } else {
            return force_low_one<A, G>(P0, V, i, cross);
        }
    };
    if constexpr (G::kWarp) {
        for_each_particle<G>(n, [&](int i) {
            if (one(i) && G::leader()) atomicAdd(&V.split_tile[i / kSplitTile], 1u);
        });
    } else {
        const int lane = threadIdx.x & 31;
        for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
            const int i = base + threadIdx.x;
            const bool flag = i < n && one(i);
            const unsigned m = __ballot_sync(0xffffffffu, flag);
            if (lane == 0 && m) atomicAdd(&V.split_tile[(base + (threadIdx.x & ~31)) / kSplitTile], __popc(m));
        }
    }
}

// ---------------------------------------------------------------------------
// High-res force + integrate + tether: computeParticleAccelerationAndAdvanceHigh
// (WCSPHSolver.cu:1867-2033) and adjustOrInjectTransientHighD (1097-1172).
// Reads see the pre-step state (the reference integrates in place, a data race);
// low-res states are read after this step's split marks, as in the reference.
// ---------------------------------------------------------------------------
template <class A, class G>
__device__ __forceinline__ void force_high_one(const Params& P, const StepView& V, int i) {
    const ScaleView& H = V.H;
    const ScaleView& L = V.L;
    float2 p = H.pos[i], v = H.vel[i];
    const unsigned s = H.st[i];
    const float dens = H.dens[i], qi = H.q[i];
    PairTerms fh{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};  // (acc, accT)
    float2 pij = make_float2(0.f, 0.f);
    float x = 0.0f;
    int csx, csy, cex, cey;
    grid_coord_s<1>(P, p.x, p.y, -P.rh, csx, csy);
    grid_coord_s<1>(P, p.x, p.y, P.rh, cex, cey);
    {
        const auto test = [&](int k) {
            if (!lamHH(s, H.st[k])) return false;
            pij = sub(p, H.pos[k]);
            x = sq(pij);
            return x != 0.0f && x <= P.Tlt_rh;
        };
        const auto term = [&](int j) {
            return A::template pair<kHHigh>(P, pij, x, sub(v, H.vel[j]), qi, H.q[j], dens, H.dens[j]);
        };
        const auto test_n = [&](const NbrState& n) {
            if (!lamHH(s, n.st)) return false;
            pij = sub(p, n.pos);
            x = sq(pij);
            return x != 0.0f && x <= P.Tlt_rh;
        };
        const auto term_n = [&](const NbrState& n) {
            return A::template pair<kHHigh>(P, pij, x, sub(v, n.vel), qi, n.q, dens, n.dens);
        };
        list_or_walk<G>(H, i, test_n, term_n, add_terms, fh,
                        [&] { G::window(H.off + P.cbH, P.dimH[0], csx, cex, csy, cey, test, term, add_terms, fh); });
    }
    grid_coord_s<0>(P, p.x, p.y, -P.r, csx, csy);
    grid_coord_s<0>(P, p.x, p.y, P.r, cex, cey);
    PairTerms fl{make_float2(0.f, 0.f), fh.t};  // (accL, accT): the sigma sum continues
    // A state-1 child pairs only with low-res entries in state 0 (lambda_HL and
    // notDeleted); a row of the window whose cells the low-res force did not stamp
    // in this step holds none, and is skipped.
    const bool odd = (s & 1u) != 0u;
    const uint8_t stamp = static_cast<uint8_t>(V.cnt->steps);
    G::window_if(
        L.off + P.cbL, P.dimL[0], csx, cex, csy, cey,
        [&](int row) {
            if (!odd) return true;
            const uint8_t* f = L.cflag + P.cbL + row;
            for (int cx = csx; cx <= cex; ++cx)
                if (f[cx] == stamp) return true;
            return false;
        },
        [&](int k) {
            const unsigned sj = L.nst[k];  // low-res states after this step's split marks
            if (!(lamHL(s, sj) && notDeleted(sj))) return false;
            pij = sub(p, L.pos[k]);
            x = sq(pij);
            return x != 0.0f && x <= P.Tlt_r;
        },
        [&](int j) {
            return A::template pair<kHCross>(P, pij, x, sub(v, L.vel[j]), qi, L.q[j], dens, L.dens[j]);
        },
        add_terms, fl);
    const float2 accB = wall_sum<A, G, 1>(P, V, p, csx, cex, csy, cey, P.Tle_rh, P.cBH);
    float2 acc = fh.a, accL = fl.a;
    const float2 accT = fl.t;
    acc.x *= -P.mH;
    acc.y *= -P.mH;
    accL.x *= -P.mL;
    accL.y *= -P.mL;
    acc.x -= P.sigma * accT.x;
    acc.y -= P.sigma * accT.y;
    acc.x += accL.x;
    acc.y += accL.y;
    acc.x += accB.x;
    acc.y += accB.y;
    acc.y -= P.g;
    v.x += P.dt * acc.x;
    v.y += P.dt * acc.y;
    p.x += P.dt * v.x;
    p.y += P.dt * v.y;
    // tether to the parent after the parent's advance (adjustPosition, 1007-1022);
    // with TSS_FLAG_MERGE the children of a parent that merged back in this step
    // are removed instead
    const int id = H.id[i];
    const int parent = id >> 2;
    bool drop = false;
    if (parent >= 0 && parent < P.slotsL) {
        const int pi = L.map[parent];
        drop = P.merge && pi >= 0 && L.st[pi] == 1 && L.nst[pi] == 0;
        if (pi >= 0 && L.st[pi] == 1 && !drop) {
            const float2 pl = L.npos[pi];
            const float2 pji = sub(p, pl);
            const float dist = vnorm(pji);
            const float lim = fminf(dist, L.tr[pi]);  // the parent's radius, from the low-res force
            if (!(P.tether_guard && dist == 0.0f)) {  // guarded: a child on its parent stays there
                p.x = pl.x + lim / dist * pji.x;
                p.y = pl.y + lim / dist * pji.y;
            }
        }
    }
    if (!G::leader()) return;
    H.acc[i] = acc;
    if (!isfinite(acc.x) || !isfinite(acc.y)) atomicOr(&V.cnt->err, kErrNumeric);
    H.npos[i] = p;
    H.nvel[i] = v;
    H.nst[i] = static_cast<uint8_t>(drop ? 2u : s);
    H.nid[i] = id;
    if (drop) {  // out of the next grid build, and of the slot map
        H.gkey[i] = -1;
        H.map[id] = -1;
        atomicAdd(&V.cnt->n_drop, 1);
    } else {
        grid_key(H.gcount, H.gkey, H.grank, H.gtile, i, P.cbH + cell_hash_s<1>(P, p));
    }
    if (H.ndens) {
        H.ndens[i] = dens;
        H.npres[i] = H.pres[i];
    }
}

// Register budgets measured per form.  The batched form reads each particle's
// parameters from the scene table: at 40 registers it spilled ~300 bytes, at 48 a
// third of that, at 64 (four blocks per SM) nothing -- as fast as 48 on a batch of
// 512 mixed scenes and 15 % faster on a batch of one 162k-particle scene.  The
// single-scene form at 48 registers (five blocks) spills 64 bytes instead of 120
// at 40 and measured 3-4 % faster.  In the tolerance arithmetic the single-scene
// form needs no spill at 40 registers (six blocks per SM) and is 3.8 % faster there
// on the developed 1M dam break (0.159 -> 0.153 ms).  The batched form in the
// tolerance arithmetic runs five blocks per SM (48 registers, 28 bytes spilled):
// 4 % faster than four on the 512-scene batch (2.16 against 2.26 ms), where the
// exact arithmetic's batched form was 8 % slower at five.
template <bool B, class G, class A>
__global__ void __launch_bounds__(256, B ? (A::kFast ? 5 : 4) : (A::kFast ? 6 : 5)) k_force_high(Params P0, StepView V) {
    for_each_particle<G>(V.cnt->cur[1], [&](int i) {
        if constexpr (B) {
            const Params& P = V.table[V.scH[i]];
            force_high_one<A, G>(P, V, i);
        } else {
            force_high_one<A, G>(P0, V, i);
        }
    });
}

// ---------------------------------------------------------------------------
// Host side: launch gather g (0 high-res density, 1 low-res density, 2 low-res
// force, 3 high-res force) in arithmetic A, and its occupancy.
// ---------------------------------------------------------------------------
template <class A, bool B, class G>
void launch_gather_bg(int g, int blocks, int threads, cudaStream_t s, const Params& P, const StepView& V) {
    switch (g) {
        case 0:
            k_density_high<B, G, A><<<blocks, threads, 0, s>>>(P, V);
            break;
        case 1:
            k_density_low<B, G, A><<<blocks, threads, 0, s>>>(P, V);
            break;
        case 2:
            k_force_low<B, G, A><<<blocks, threads, 0, s>>>(P, V);
            break;
        case 3:
            k_force_high<B, G, A><<<blocks, threads, 0, s>>>(P, V);
            break;
        default:
            break;
    }
}

template <class A>
void launch_gather_a(int g, bool batched, bool warp, int blocks, int threads, cudaStream_t s, const Params& P,
                     const StepView& V) {
    if (batched) {
        if (warp)
            launch_gather_bg<A, true, PerWarp>(g, blocks, threads, s, P, V);
        else
            launch_gather_bg<A, true, PerThread>(g, blocks, threads, s, P, V);
    } else {
        if (warp)
            launch_gather_bg<A, false, PerWarp>(g, blocks, threads, s, P, V);
        else
            launch_gather_bg<A, false, PerThread>(g, blocks, threads, s, P, V);
    }
}

template <class K>
int occupancy_of(K kernel, int threads) {
    int n = 0;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, 0) == cudaSuccess ? n : 0;
}

template <class A, bool B, class G>
int gather_occupancy_bg(int g, int threads) {
    switch (g) {
        case 0:
            return occupancy_of(k_density_high<B, G, A>, threads);
        case 1:
            return occupancy_of(k_density_low<B, G, A>, threads);
        case 2:
            return occupancy_of(k_force_low<B, G, A>, threads);
        case 3:
            return occupancy_of(k_force_high<B, G, A>, threads);
        default:
            return 0;
    }
}

template <class A>
int gather_occupancy_a(int g, bool batched, bool warp, int threads) {
    if (batched)
        return warp ? gather_occupancy_bg<A, true, PerWarp>(g, threads) : gather_occupancy_bg<A, true, PerThread>(g, threads);
    return warp ? gather_occupancy_bg<A, false, PerWarp>(g, threads) : gather_occupancy_bg<A, false, PerThread>(g, threads);
}

}  // namespace tss
