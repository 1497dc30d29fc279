// tss_oracle.cpp -- CPU ORACLE for the two-scale WCSPH step.  TEST INFRASTRUCTURE ONLY.
//
// This file restates, on the CPU, the step of the reference's WCSPHSolver::AdvanceTS
// (TwoScale2D/WCSPHSolver.cu:2726-2810) one kernel at a time, templated on the float
// type: instantiated with float it follows the reference's FP32 operation order
// exactly (compile with -ffp-contract=off), with double it is the FP64 error
// reference.  Only the test suite, the smoke check and bench.py's CPU-baseline leg
// load it; the product library never does.
//
// Semantics, with the reference line each part follows:
//  * cell hash            WCSPHSolver.cu:241-323   (truncate toward zero, clamp)
//  * list order           stable sort by cell of an id-ascending list = (cell, id)
//                         order; the reference's order within a cell depends on
//                         atomicAdd append order (1826, 2030, 1135) and is not
//                         deterministic, any fixed order is one of its schedules
//  * kernels W, dW, wall  WCSPHSolver.cu:66-239, coefficients Bind 2559-2590
//  * high density         1426-1516 (+402-474); Q1 compat switch for 1483-1510
//  * low density          1342-1424 (+335-400)
//  * low force + split    1648-1865 (+476-660, 956-1005), advance 1604-1646 fused
//  * high force+integrate 1867-2033 (+662-737, 786-885); Jacobi: reads see the
//                         pre-step state (the reference writes in place, 2020-2027)
//  * tether               1097-1172 (+1007-1022)
//  * relaxation           TwoScale2D-master/TwoScale2D/WCSPHSolver.cu:2380-2446,
//                         density 1133-1217 (+351-379), force 1499-1622
//                         (= TwoScale2D/WCSPHSolver.cu:2035-2158, +739-784, 887-954)
//  * uninitialised accL   (1919-1921) is taken as zero.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/tss.h"

namespace {

const double kPi = 3.14159265358979323846;  // WCSPHSolver.cu:19

// float -> int as CUDA's cvt.rzi.s32: truncate toward zero, saturate, NaN -> 0.
template <class T>
inline int f2i(T v) {
    if (v != v) return 0;
    if (v >= T(2147483647.0)) return INT_MAX;
    if (v <= T(-2147483648.0)) return INT_MIN;
    return static_cast<int>(v);
}

struct Grid {
    double ox, oy;  // not used in arithmetic; the typed copies below are
    int dimx = 1, dimy = 1;
    int ncells() const { return dimx * dimy; }
};

template <class T>
struct V2 {
    T x, y;
};

template <class T>
struct Consts {
    T ox, oy;
    int dimL[2], dimH[2];
    T r, rh, rho0, B, cs, alpha, sigma, dt, g;
    T CL, GL, CH, GH;  // kernel / gradient coefficients, low & high
    T mL, mH, mB;
    T cBL, cBH;  // wall mass ratios mB/(mL+mB), mB/(mH+mB)
    T relax_dt;
    T roi[4];
    T roi_vdt[2];  // ROI displacement per step (roi_velocity * dt)
    int relax_iters;
    bool q1;
    bool merge;    // TSS_FLAG_MERGE: split parents outside the ROI merge back
    bool tether_guard;  // TSS_FLAG_TETHER_GUARD: no 0/0 when a child sits on its parent
    bool older_place;   // TSS_FLAG_OLDER_PLACEMENT: children at +-DIR_LEN*r (older snapshot 840-850)
};

// computeGridCoordinate(pos, offset), WCSPHSolver.cu:265-289.
template <class T>
inline void coord(T px, T py, T off, T ox, T oy, T cell, const int dim[2], int& cx, int& cy) {
    cx = f2i(((px + off) - ox) / cell);
    cy = f2i(((py + off) - oy) / cell);
    cx = std::min(std::max(0, cx), dim[0] - 1);
    cy = std::min(std::max(0, cy), dim[1] - 1);
}

// evaluateM4Kernel / evaluateM4KernelHigh, WCSPHSolver.cu:116-160.
template <class T>
inline T W(T d, T rad, T C) {
    T q = d * T(2) / rad;
    if (q < T(1)) {
        T a = T(2) - q, b = T(1) - q;
        return C * (a * a * a - T(4) * b * b * b);
    } else if (q < T(2)) {
        T a = T(2) - q;
        return C * a * a * a;
    }
    return T(0);
}

// evaluateGradientM4Kernel(High), WCSPHSolver.cu:162-239.
template <class T>
inline V2<T> dW(V2<T> x, T d, T rad, T G) {
    T q = d * T(2) / rad;
    if (q < T(1)) {
        T a = T(2) - q, b = T(1) - q;
        T c = G * (a * a - T(4) * b * b) / d;
        return {c * x.x, c * x.y};
    } else if (q < T(2)) {
        T a = T(2) - q;
        T c = G * a * a / d;
        return {c * x.x, c * x.y};
    }
    return {T(0), T(0)};
}

// evaluateBoundaryForceWeight(High), WCSPHSolver.cu:66-114.
template <class T>
inline T gamma_wall(T d, T rad, T cs) {
    T q = d * T(2) / rad;
    T c = T(0.02f) * cs * cs / (d * d);
    if (q < T(2) / T(3)) return c * T(2) / T(3);
    if (q < T(1)) return c * (T(2) * q - T(3) / T(2) * q * q);
    if (q < T(2)) {
        T a = T(2) - q;
        return c * T(0.5f) * a * a;
    }
    return T(0);
}

template <class T>
inline T norm2(V2<T> v) {
    return std::sqrt(v.x * v.x + v.y * v.y);
}

template <class T>
inline T tait(T dens, const Consts<T>& k) {
    T a = dens / k.rho0;
    T a3 = a * a * a;
    return k.B * (a3 * a3 * a - T(1));
}

const float kLamLH[4] = {1.f, 0.f, 1.f, 0.f};  // updateDensityCellComplement 377, updateAccCellComplement 602
const float kLamHH[4] = {1.f, 0.f, 1.f, 1.f};  // updateDensityCellHigh 414, updateAccCellHigh 681
const float kLamHL[4] = {1.f, 1.f, 1.f, 0.f};  // updateDensityCellComplementHigh 451, 808
const float kDel[3] = {1.f, 1.f, 0.f};         // "deleted" table 500, 809
inline int lam_idx(uint8_t si, uint8_t sj) { return ((si & 1) << 1) | (sj & 1); }
inline float del_w(uint8_t s) { return s < 3 ? kDel[s] : 0.f; }

// One scale's particles: list-order state plus this step's sorted arrays.
template <class T>
struct Scale {
    // list order (input of the next step)
    std::vector<int32_t> id;
    std::vector<V2<T>> pos, vel;
    std::vector<uint8_t> st;
    std::vector<T> dens, pres;
    // sorted order (this step)
    std::vector<int32_t> s_src, s_id, off;
    std::vector<V2<T>> s_pos, s_vel, s_acc;
    std::vector<uint8_t> s_st;
    std::vector<T> s_dens, s_pres, s_q;  // q = p / rho^2
    std::vector<T> s_scale;              // |summands| of each acceleration (want_scale only)
    std::vector<int32_t> map;            // slot id -> sorted index, -1 if absent
    int n() const { return (int)id.size(); }
};

// Stable order by (cell, id): bucket by cell in input order, then sort each bucket
// by id.  Dense offsets off[c] (C+1 entries).
template <class T>
void grid_order(int n, const V2<T>* pos, const int32_t* id, T ox, T oy, T cell, const int dim[2],
                std::vector<int32_t>& order, std::vector<int32_t>& off) {
    const int C = dim[0] * dim[1];
    std::vector<int32_t> hash(n);
    for (int i = 0; i < n; ++i) {
        int cx, cy;
        coord<T>(pos[i].x, pos[i].y, T(0), ox, oy, cell, dim, cx, cy);
        hash[i] = cy * dim[0] + cx;  // computeHash, WCSPHSolver.cu:291-296
    }
    off.assign(C + 1, 0);
    for (int i = 0; i < n; ++i) off[hash[i] + 1]++;
    for (int c = 0; c < C; ++c) off[c + 1] += off[c];
    order.assign(n, 0);
    std::vector<int32_t> fill(off.begin(), off.end() - 1);
    for (int i = 0; i < n; ++i) order[fill[hash[i]]++] = i;
    for (int c = 0; c < C; ++c) {
        int a = off[c], b = off[c + 1];
        if (b - a > 1)
            std::sort(order.begin() + a, order.begin() + b,
                      [&](int32_t u, int32_t v) { return id[u] < id[v]; });
    }
}

template <class T>
class Oracle {
public:
    Consts<T> k;
    tss_config cfg;
    int slotsL = 0, slotsH = 0, capH = 0;
    Scale<T> L, H;
    // walls, sorted by (low cell, id) once
    std::vector<V2<T>> wall;
    std::vector<int32_t> wall_off;
    std::vector<int32_t> fresh;  // low-res parents split last step
    std::vector<int32_t> split;  // parents split this step
    int overflow = 0;
    long long steps_done = 0;    // the ROI of step k is roi + k * roi_vdt
    int removed = 0;             // children removed by merges in the last step

    Oracle(const tss_config& c, float mL, float mH, float mB, int nL_slots, int cap_high,
           int n_wall, const float* wall_pos)
        : cfg(c) {
        k.ox = T(c.domain_origin[0]);
        k.oy = T(c.domain_origin[1]);
        k.dimL[0] = c.dims_low[0];
        k.dimL[1] = c.dims_low[1];
        k.dimH[0] = c.dims_high[0];
        k.dimH[1] = c.dims_high[1];
        k.r = T(c.r_low);
        k.rh = T(c.r_high);
        k.rho0 = T(c.rest_density);
        k.B = T(c.tait_b);
        k.cs = T(c.speed_sound);
        k.alpha = T(c.alpha);
        k.sigma = T(c.tension);
        k.dt = T(c.dt);
        k.g = T(c.gravity);
        // Bind(): coefficients evaluated in double then stored as float (2559-2590).
        double r = c.r_low, rh = c.r_high;
        k.CL = T(20.0 / (14.0 * kPi * r * r));
        k.GL = T(-120.0 / (14.0 * kPi * r * r * r));
        k.CH = T(20.0 / (14.0 * kPi * rh * rh));
        k.GH = T(-120.0 / (14.0 * kPi * rh * rh * rh));
        k.mL = T(mL);
        k.mH = T(mH);
        k.mB = T(mB);
        k.cBL = k.mB / (k.mL + k.mB);
        k.cBH = k.mB / (k.mH + k.mB);
        k.relax_dt = k.dt / T(c.relax_dt_div);
        for (int i = 0; i < 4; ++i) k.roi[i] = T(c.roi[i]);
        k.roi_vdt[0] = T(c.roi_velocity[0]) * T(c.dt);
        k.roi_vdt[1] = T(c.roi_velocity[1]) * T(c.dt);
        k.relax_iters = c.relax_iters;
        k.q1 = (c.flags & TSS_FLAG_Q1_COMPAT) != 0;
        k.merge = (c.flags & TSS_FLAG_MERGE) != 0;
        k.tether_guard = (c.flags & TSS_FLAG_TETHER_GUARD) != 0;
        k.older_place = (c.flags & TSS_FLAG_OLDER_PLACEMENT) != 0;
        slotsL = nL_slots;
        slotsH = 4 * nL_slots;
        capH = cap_high;
        wall.resize(n_wall);
        std::vector<int32_t> wid(n_wall);
        for (int i = 0; i < n_wall; ++i) {
            wall[i] = {T(wall_pos[2 * i]), T(wall_pos[2 * i + 1])};
            wid[i] = i;
        }
        // initBoundaries (3205-3238): iota ids, hash on the LOW grid, stable sort.
        std::vector<int32_t> order;
        grid_order<T>(n_wall, wall.data(), wid.data(), k.ox, k.oy, k.r, k.dimL, order, wall_off);
        std::vector<V2<T>> w2(n_wall);
        for (int i = 0; i < n_wall; ++i) w2[i] = wall[order[i]];
        wall.swap(w2);
    }

    void build(Scale<T>& S, T cell, const int dim[2], int slots, bool carry) {
        const int n = S.n();
        grid_order<T>(n, S.pos.data(), S.id.data(), k.ox, k.oy, cell, dim, S.s_src, S.off);
        S.s_id.resize(n);
        S.s_pos.resize(n);
        S.s_vel.resize(n);
        S.s_st.resize(n);
        S.s_acc.assign(n, {T(0), T(0)});
        S.s_dens.assign(n, T(0));
        S.s_pres.assign(n, T(0));
        S.s_q.assign(n, T(0));
        S.map.assign(slots, -1);
        for (int i = 0; i < n; ++i) {
            int s = S.s_src[i];
            S.s_id[i] = S.id[s];
            S.s_pos[i] = S.pos[s];
            S.s_vel[i] = S.vel[s];
            S.s_st[i] = S.st[s];
            if (carry) {
                S.s_dens[i] = S.dens[s];
                S.s_pres[i] = S.pres[s];
            }
            S.map[S.id[s]] = i;
        }
    }

    // ---- relaxation of the children created last step (older tree 2380-2446) ----
    void relax() {
        std::vector<int32_t> kids;
        for (int p : fresh)
            for (int c = 0; c < 4; ++c) {
                int slot = 4 * p + c;
                int idx = (slot >= 0 && slot < slotsH) ? H.map[slot] : -1;
                if (idx >= 0) kids.push_back(idx);
            }
        const int nk = (int)kids.size();
        std::vector<V2<T>> npos(nk), nvel(nk);
        for (int it = 0; it < k.relax_iters; ++it) {
            // computeParticleDensityPressureHighRelax (older 1133-1217)
#pragma omp parallel for schedule(static)
            for (int f = 0; f < nk; ++f) {
                int i = kids[f];
                V2<T> p = H.s_pos[i];
                T d = 0, dl = 0;
                int csx, csy, cex, cey;
                coord<T>(p.x, p.y, -k.rh, k.ox, k.oy, k.rh, k.dimH, csx, csy);
                coord<T>(p.x, p.y, k.rh, k.ox, k.oy, k.rh, k.dimH, cex, cey);
                for (int cy = csy; cy <= cey; ++cy)
                    for (int cx = csx; cx <= cex; ++cx) {
                        int h = cy * k.dimH[0] + cx;
                        for (int j = H.off[h]; j < H.off[h + 1]; ++j) {
                            V2<T> pij{p.x - H.s_pos[j].x, p.y - H.s_pos[j].y};
                            T dist = norm2(pij);
                            if (dist <= k.rh) d += W(dist, k.rh, k.CH);
                        }
                    }
                coord<T>(p.x, p.y, -k.rh, k.ox, k.oy, k.r, k.dimL, csx, csy);
                coord<T>(p.x, p.y, k.rh, k.ox, k.oy, k.r, k.dimL, cex, cey);
                for (int cy = csy; cy <= cey; ++cy)
                    for (int cx = csx; cx <= cex; ++cx) {
                        int h = cy * k.dimL[0] + cx;
                        for (int j = L.off[h]; j < L.off[h + 1]; ++j) {
                            V2<T> pij{p.x - L.s_pos[j].x, p.y - L.s_pos[j].y};
                            T dist = norm2(pij);
                            if (dist <= k.rh) dl += W(dist, k.rh, k.CH);
                        }
                    }
                d *= k.mH;
                dl *= k.mL;
                d += dl;
                H.s_dens[i] = d;
                H.s_pres[i] = tait(d, k);
            }
            // computeParticleAccelerationAndAdvanceHighRelax (2035-2158)
#pragma omp parallel for schedule(static)
            for (int f = 0; f < nk; ++f) {
                int i = kids[f];
                V2<T> p = H.s_pos[i], v = H.s_vel[i];
                T dens = H.s_dens[i], pre = H.s_pres[i];
                T dens2 = dens * dens;
                V2<T> acc{0, 0}, accL{0, 0}, accB{0, 0};
                int csx, csy, cex, cey;
                coord<T>(p.x, p.y, -k.rh, k.ox, k.oy, k.rh, k.dimH, csx, csy);
                coord<T>(p.x, p.y, k.rh, k.ox, k.oy, k.rh, k.dimH, cex, cey);
                for (int cy = csy; cy <= cey; ++cy)
                    for (int cx = csx; cx <= cex; ++cx) {
                        int h = cy * k.dimH[0] + cx;
                        for (int j = H.off[h]; j < H.off[h + 1]; ++j) {
                            V2<T> pij{p.x - H.s_pos[j].x, p.y - H.s_pos[j].y};
                            T dist = norm2(pij);
                            if (dist != T(0) && dist < k.rh) {
                                T dj = H.s_dens[j];
                                T coeff = pre / dens2 + H.s_pres[j] / (dj * dj);
                                V2<T> g = dW(pij, dist, k.rh, k.GH);
                                acc.x += coeff * g.x;
                                acc.y += coeff * g.y;
                            }
                        }
                    }
                coord<T>(p.x, p.y, -k.rh, k.ox, k.oy, k.r, k.dimL, csx, csy);
                coord<T>(p.x, p.y, k.rh, k.ox, k.oy, k.r, k.dimL, cex, cey);
                for (int cy = csy; cy <= cey; ++cy)
                    for (int cx = csx; cx <= cex; ++cx) {
                        int h = cy * k.dimL[0] + cx;
                        for (int j = L.off[h]; j < L.off[h + 1]; ++j) {
                            V2<T> pij{p.x - L.s_pos[j].x, p.y - L.s_pos[j].y};
                            T dist = norm2(pij);
                            if (dist != T(0) && dist < k.rh) {
                                T dj = L.s_dens[j];
                                T coeff = pre / dens2 + L.s_pres[j] / (dj * dj);
                                V2<T> g = dW(pij, dist, k.rh, k.GH);
                                accL.x += coeff * g.x;
                                accL.y += coeff * g.y;
                            }
                        }
                        for (int b = wall_off[h]; b < wall_off[h + 1]; ++b) {
                            V2<T> pik{p.x - wall[b].x, p.y - wall[b].y};
                            T dist = norm2(pik);
                            T gm = gamma_wall(dist, k.rh, k.cs);
                            accB.x += k.cBH * gm * pik.x;
                            accB.y += k.cBH * gm * pik.y;
                        }
                    }
                acc.x *= -k.mH;
                acc.y *= -k.mH;
                accL.x *= -k.mL;
                accL.y *= -k.mL;
                acc.x += accL.x;
                acc.y += accL.y;
                acc.x += accB.x;
                acc.y += accB.y;
                v.x += k.relax_dt * acc.x;
                v.y += k.relax_dt * acc.y;
                p.x += k.relax_dt * v.x;
                p.y += k.relax_dt * v.y;
                npos[f] = p;
                nvel[f] = v;
            }
            for (int f = 0; f < nk; ++f) {
                H.s_pos[kids[f]] = npos[f];
                H.s_vel[kids[f]] = nvel[f];
            }
        }
    }

    // ---- high-res density, WCSPHSolver.cu:1426-1516 ----
    void density_high() {
        const int n = H.n();
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V2<T> p = H.s_pos[i];
            uint8_t s = H.s_st[i];
            T d = 0, dl = 0;
            int csx, csy, cex, cey;
            coord<T>(p.x, p.y, -k.rh, k.ox, k.oy, k.rh, k.dimH, csx, csy);
            coord<T>(p.x, p.y, k.rh, k.ox, k.oy, k.rh, k.dimH, cex, cey);
            for (int cy = csy; cy <= cey; ++cy)
                for (int cx = csx; cx <= cex; ++cx) {
                    int h = cy * k.dimH[0] + cx;
                    for (int j = H.off[h]; j < H.off[h + 1]; ++j) {
                        float lam = kLamHH[lam_idx(s, H.s_st[j])];
                        if (lam == 0.f) continue;
                        V2<T> pij{p.x - H.s_pos[j].x, p.y - H.s_pos[j].y};
                        T dist = norm2(pij);
                        if (dist <= k.rh) d += T(lam) * (W(dist, k.r, k.CL) + W(dist, k.rh, k.CH)) / T(2);
                    }
                }
            coord<T>(p.x, p.y, -k.r, k.ox, k.oy, k.r, k.dimL, csx, csy);
            coord<T>(p.x, p.y, k.r, k.ox, k.oy, k.r, k.dimL, cex, cey);
            for (int cy = csy; cy <= cey; ++cy)
                for (int cx = csx; cx <= cex; ++cx) {
                    int h = cy * k.dimL[0] + cx;
                    for (int t = L.off[h]; t < L.off[h + 1]; ++t) {
                        if (k.q1) {
                            // The reference reads the HIGH sorted list at a LOW-grid range;
                            // beyond n_high that list still holds its initial identity.
                            V2<T> pj{0, 0};
                            uint8_t sj = 0;
                            if (t < n) {
                                pj = H.s_pos[t];
                                sj = H.s_st[t];
                            } else {
                                int idx = t < slotsH ? H.map[t] : -1;
                                if (idx >= 0) {
                                    pj = H.s_pos[idx];
                                    sj = H.s_st[idx];
                                }
                            }
                            float lam = kLamHL[lam_idx(s, sj)];
                            if (lam == 0.f) continue;
                            V2<T> pij{p.x - pj.x, p.y - pj.y};
                            T dist = norm2(pij);
                            if (dist <= k.rh) d += T(lam) * (W(dist, k.r, k.CL) + W(dist, k.rh, k.CH)) / T(2);
                        } else {
                            float lam = kLamHL[lam_idx(s, L.s_st[t])];
                            if (lam == 0.f) continue;
                            V2<T> pij{p.x - L.s_pos[t].x, p.y - L.s_pos[t].y};
                            T dist = norm2(pij);
                            if (dist <= k.rh) dl += T(lam) * (W(dist, k.r, k.CL) + W(dist, k.rh, k.CH)) / T(2);
                        }
                    }
                }
            d *= k.mH;
            dl *= k.mL;
            d += dl;
            H.s_dens[i] = d;
            T pr = tait(d, k);
            H.s_pres[i] = pr;
            H.s_q[i] = pr / (d * d);
        }
    }

    // ---- low-res density, WCSPHSolver.cu:1342-1424 ----
    void density_low() {
        const int n = L.n();
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V2<T> p = L.s_pos[i];
            uint8_t s = L.s_st[i];
            T d = 0, dh = 0;
            int csx, csy, cex, cey;
            coord<T>(p.x, p.y, -k.r, k.ox, k.oy, k.r, k.dimL, csx, csy);
            coord<T>(p.x, p.y, k.r, k.ox, k.oy, k.r, k.dimL, cex, cey);
            for (int cy = csy; cy <= cey; ++cy)
                for (int cx = csx; cx <= cex; ++cx) {
                    int h = cy * k.dimL[0] + cx;
                    for (int j = L.off[h]; j < L.off[h + 1]; ++j) {
                        V2<T> pij{p.x - L.s_pos[j].x, p.y - L.s_pos[j].y};
                        T dist = norm2(pij);
                        if (dist <= k.r) d += (W(dist, k.r, k.CL) + W(dist, k.rh, k.CH)) / T(2);
                    }
                }
            coord<T>(p.x, p.y, -k.r, k.ox, k.oy, k.rh, k.dimH, csx, csy);
            coord<T>(p.x, p.y, k.r, k.ox, k.oy, k.rh, k.dimH, cex, cey);
            for (int cy = csy; cy <= cey; ++cy)
                for (int cx = csx; cx <= cex; ++cx) {
                    int h = cy * k.dimH[0] + cx;
                    for (int j = H.off[h]; j < H.off[h + 1]; ++j) {
                        float lam = kLamLH[lam_idx(s, H.s_st[j])];
                        if (lam == 0.f) continue;
                        V2<T> pij{p.x - H.s_pos[j].x, p.y - H.s_pos[j].y};
                        T dist = norm2(pij);
                        if (dist <= k.r) dh += T(lam) * (W(dist, k.r, k.CL) + W(dist, k.rh, k.CH)) / T(2);
                    }
                }
            d *= k.mL;
            dh *= k.mH;
            T rho = d + dh;
            L.s_dens[i] = rho;
            T pr = tait(rho, k);
            L.s_pres[i] = pr;
            L.s_q[i] = pr / (rho * rho);
        }
    }

    // one pair of the force sums (updateAccCell* bodies)
    inline void pair_force(V2<T> pij, T dist, V2<T> vij, T qi, T qj, T densi, T densj, T h, T lw,
                           V2<T>& acc, V2<T>& accT) const {
        T coeff = qi + qj;
        T dvp = vij.x * pij.x + vij.y * pij.y;
        if (dvp < T(0)) coeff -= dvp / (dist * dist + T(0.01f) * h * h) * T(2) * h * k.alpha * k.cs / (densi + densj);
        V2<T> gI = dW(pij, dist, k.r, k.GL);
        V2<T> gJ = dW(pij, dist, k.rh, k.GH);
        acc.x += lw * coeff * (gI.x + gJ.x) / T(2);
        acc.y += lw * coeff * (gI.y + gJ.y) / T(2);
        T w = W(dist, k.r, k.CL);
        T w2 = W(dist, k.rh, k.CH);
        accT.x += lw * pij.x * (w + w2) / T(2);
        accT.y += lw * pij.y * (w + w2) / T(2);
    }

    // The error scale of an acceleration, against which a per-step tolerance on it
    // is stated: the sum of the magnitudes of its summands (m |pressure/viscosity
    // term| over both scales' pairs, sigma |tension term|, |wall term|, g), where a
    // pressure term's magnitude also counts how far it moves when the two densities
    // move by their own relative amount (kappa = |d(p/rho^2)/d rho| rho, from the
    // Tait equation).  Each summand carries its own rounding, and near rest density
    // the Tait equation turns a density's last-place rounding into a large relative
    // change of its pressure, so an FP32 evaluation is only accurate to a few units
    // of this scale however small the acceleration: a result within tol * scale is
    // the exact sum for densities and summands each within tol relative.  Computed
    // only when want_scale is set (a separate pass; the step's results do not
    // depend on it).
    bool want_scale = false;
    inline T eos_kappa(T q, T dens) const {
        const T a = dens / k.rho0;
        const T a3 = a * a * a;
        return std::fabs(T(7) * k.B * a3 * a3 / (k.rho0 * dens) - T(2) * q / dens);
    }
    inline void pair_mag(V2<T> pij, T dist, V2<T> vij, T qi, T qj, T densi, T densj, T h, T lw, T& ma,
                         T& mt) const {
        T visc = T(0);
        T dvp = vij.x * pij.x + vij.y * pij.y;
        if (dvp < T(0)) visc = dvp / (dist * dist + T(0.01f) * h * h) * T(2) * h * k.alpha * k.cs / (densi + densj);
        const T cmag = std::fabs(qi) + std::fabs(qj) + std::fabs(visc) + eos_kappa(qi, densi) + eos_kappa(qj, densj);
        V2<T> gI = dW(pij, dist, k.r, k.GL);
        V2<T> gJ = dW(pij, dist, k.rh, k.GH);
        ma += std::fabs(lw) * cmag * std::hypot(gI.x + gJ.x, gI.y + gJ.y) / T(2);
        mt += std::fabs(lw) * std::hypot(pij.x, pij.y) * std::fabs(W(dist, k.r, k.CL) + W(dist, k.rh, k.CH)) / T(2);
    }

    // ---- low-res force, predicted advance, split (1648-1865, 1604-1646, 956-1005) ----
    std::vector<uint8_t> nxt_stL;
    std::vector<V2<T>> nxt_posL, nxt_velL;
    void force_low() {
        const int n = L.n();
        nxt_stL.assign(L.s_st.begin(), L.s_st.end());
        nxt_posL.resize(n);
        nxt_velL.resize(n);
        std::vector<uint8_t> flag(n, 0);
        if (want_scale) L.s_scale.assign(n, T(0));
        const T hx = (k.r + k.rh) / T(2);
        // the region of interest of this step (a rectangle moving by roi_vdt per step)
        const T kf = T(steps_done);
        const T rx0 = k.roi[0] + kf * k.roi_vdt[0], rx1 = k.roi[2] + kf * k.roi_vdt[0];
        const T ry0 = k.roi[1] + kf * k.roi_vdt[1], ry1 = k.roi[3] + kf * k.roi_vdt[1];
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V2<T> p = L.s_pos[i], v = L.s_vel[i];
            uint8_t s = L.s_st[i];
            T dens = L.s_dens[i], qi = L.s_q[i];
            V2<T> acc{0, 0}, accH{0, 0}, accT{0, 0}, accB{0, 0};
            T sa = 0, sah = 0, stn = 0, sb = 0;  // error scale (want_scale)
            int csx, csy, cex, cey;
            coord<T>(p.x, p.y, -k.r, k.ox, k.oy, k.r, k.dimL, csx, csy);
            coord<T>(p.x, p.y, k.r, k.ox, k.oy, k.r, k.dimL, cex, cey);
            for (int cy = csy; cy <= cey; ++cy)
                for (int cx = csx; cx <= cex; ++cx) {
                    int h = cy * k.dimL[0] + cx;
                    for (int j = L.off[h]; j < L.off[h + 1]; ++j) {
                        V2<T> pij{p.x - L.s_pos[j].x, p.y - L.s_pos[j].y};
                        T dist = norm2(pij);
                        if (dist != T(0) && dist < k.r) {
                            float lw = del_w(L.s_st[j]);
                            V2<T> vij{v.x - L.s_vel[j].x, v.y - L.s_vel[j].y};
                            pair_force(pij, dist, vij, qi, L.s_q[j], dens, L.s_dens[j], k.r, T(lw), acc, accT);
                            if (want_scale)
                                pair_mag(pij, dist, vij, qi, L.s_q[j], dens, L.s_dens[j], k.r, T(lw), sa, stn);
                        }
                    }
                    for (int b = wall_off[h]; b < wall_off[h + 1]; ++b) {
                        V2<T> pik{p.x - wall[b].x, p.y - wall[b].y};
                        T dist = norm2(pik);
                        T gm = gamma_wall(dist, k.r, k.cs);
                        accB.x += k.cBL * gm * pik.x;
                        accB.y += k.cBL * gm * pik.y;
                        if (want_scale) sb += std::fabs(k.cBL * gm) * std::hypot(pik.x, pik.y);
                    }
                }
            coord<T>(p.x, p.y, -k.r, k.ox, k.oy, k.rh, k.dimH, csx, csy);
            coord<T>(p.x, p.y, k.r, k.ox, k.oy, k.rh, k.dimH, cex, cey);
            for (int cy = csy; cy <= cey; ++cy)
                for (int cx = csx; cx <= cex; ++cx) {
                    int h = cy * k.dimH[0] + cx;
                    for (int j = H.off[h]; j < H.off[h + 1]; ++j) {
                        float lw = kLamLH[lam_idx(s, H.s_st[j])];
                        if (lw == 0.f) continue;
                        V2<T> pij{p.x - H.s_pos[j].x, p.y - H.s_pos[j].y};
                        T dist = norm2(pij);
                        if (dist != T(0) && dist < k.r) {
                            V2<T> vij{v.x - H.s_vel[j].x, v.y - H.s_vel[j].y};
                            pair_force(pij, dist, vij, qi, H.s_q[j], dens, H.s_dens[j], hx, T(lw), accH, accT);
                            if (want_scale)
                                pair_mag(pij, dist, vij, qi, H.s_q[j], dens, H.s_dens[j], hx, T(lw), sah, stn);
                        }
                    }
                }
            acc.x *= -k.mL;
            acc.y *= -k.mL;
            accH.x *= -k.mH;
            accH.y *= -k.mH;
            acc.x += accH.x;
            acc.y += accH.y;
            acc.x -= k.sigma * accT.x;
            acc.y -= k.sigma * accT.y;
            acc.x += accB.x;
            acc.y += accB.y;
            acc.y -= k.g;
            L.s_acc[i] = acc;
            if (want_scale) L.s_scale[i] = k.mL * sa + k.mH * sah + k.sigma * stn + sb + std::fabs(k.g);
            v.x += k.dt * acc.x;
            v.y += k.dt * acc.y;
            p.x += k.dt * v.x;
            p.y += k.dt * v.y;
            nxt_posL[i] = p;
            nxt_velL[i] = v;
            const bool in_roi = rx0 < p.x && p.x < rx1 && ry0 < p.y && p.y < ry1;
            if (s == 0 && in_roi) {
                nxt_stL[i] = 1;
                flag[i] = 1;
            } else if (k.merge && s == 1 && !in_roi) {
                nxt_stL[i] = 0;  // merge back: the children are removed below
            }
        }
        split.clear();
        for (int i = 0; i < n; ++i)
            if (flag[i]) split.push_back(i);  // sorted indices for now
    }

    // ---- high-res force + integrate + tether (1867-2033, 1097-1172) ----
    std::vector<V2<T>> nxt_posH, nxt_velH;
    void force_high() {
        const int n = H.n();
        nxt_posH.resize(n);
        nxt_velH.resize(n);
        if (want_scale) H.s_scale.assign(n, T(0));
        const T hx = (k.r + k.rh) / T(2);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V2<T> p = H.s_pos[i], v = H.s_vel[i];
            uint8_t s = H.s_st[i];
            T dens = H.s_dens[i], qi = H.s_q[i];
            V2<T> acc{0, 0}, accL{0, 0}, accT{0, 0}, accB{0, 0};
            T sa = 0, sal = 0, stn = 0, sb = 0;  // error scale (want_scale)
            int csx, csy, cex, cey;
            coord<T>(p.x, p.y, -k.rh, k.ox, k.oy, k.rh, k.dimH, csx, csy);
            coord<T>(p.x, p.y, k.rh, k.ox, k.oy, k.rh, k.dimH, cex, cey);
            for (int cy = csy; cy <= cey; ++cy)
                for (int cx = csx; cx <= cex; ++cx) {
                    int h = cy * k.dimH[0] + cx;
                    for (int j = H.off[h]; j < H.off[h + 1]; ++j) {
                        float lw = kLamHH[lam_idx(s, H.s_st[j])];
                        if (lw == 0.f) continue;
                        V2<T> pij{p.x - H.s_pos[j].x, p.y - H.s_pos[j].y};
                        T dist = norm2(pij);
                        if (dist != T(0) && dist < k.rh) {
                            V2<T> vij{v.x - H.s_vel[j].x, v.y - H.s_vel[j].y};
                            pair_force(pij, dist, vij, qi, H.s_q[j], dens, H.s_dens[j], k.rh, T(lw), acc, accT);
                            if (want_scale)
                                pair_mag(pij, dist, vij, qi, H.s_q[j], dens, H.s_dens[j], k.rh, T(lw), sa, stn);
                        }
                    }
                }
            coord<T>(p.x, p.y, -k.r, k.ox, k.oy, k.r, k.dimL, csx, csy);
            coord<T>(p.x, p.y, k.r, k.ox, k.oy, k.r, k.dimL, cex, cey);
            for (int cy = csy; cy <= cey; ++cy)
                for (int cx = csx; cx <= cex; ++cx) {
                    int h = cy * k.dimL[0] + cx;
                    for (int j = L.off[h]; j < L.off[h + 1]; ++j) {
                        uint8_t sj = nxt_stL[j];  // low states after this step's split marks
                        float lw = kLamHL[lam_idx(s, sj)] * del_w(sj);
                        if (lw == 0.f) continue;
                        V2<T> pij{p.x - L.s_pos[j].x, p.y - L.s_pos[j].y};
                        T dist = norm2(pij);
                        if (dist != T(0) && dist < k.r) {
                            V2<T> vij{v.x - L.s_vel[j].x, v.y - L.s_vel[j].y};
                            pair_force(pij, dist, vij, qi, L.s_q[j], dens, L.s_dens[j], hx, T(lw), accL, accT);
                            if (want_scale)
                                pair_mag(pij, dist, vij, qi, L.s_q[j], dens, L.s_dens[j], hx, T(lw), sal, stn);
                        }
                    }
                    for (int b = wall_off[h]; b < wall_off[h + 1]; ++b) {
                        V2<T> pik{p.x - wall[b].x, p.y - wall[b].y};
                        T dist = norm2(pik);
                        T gm = gamma_wall(dist, k.rh, k.cs);
                        accB.x += k.cBH * gm * pik.x;
                        accB.y += k.cBH * gm * pik.y;
                        if (want_scale) sb += std::fabs(k.cBH * gm) * std::hypot(pik.x, pik.y);
                    }
                }
            acc.x *= -k.mH;
            acc.y *= -k.mH;
            accL.x *= -k.mL;
            accL.y *= -k.mL;
            acc.x -= k.sigma * accT.x;
            acc.y -= k.sigma * accT.y;
            acc.x += accL.x;
            acc.y += accL.y;
            acc.x += accB.x;
            acc.y += accB.y;
            acc.y -= k.g;
            H.s_acc[i] = acc;
            if (want_scale) H.s_scale[i] = k.mH * sa + k.mL * sal + k.sigma * stn + sb + std::fabs(k.g);
            v.x += k.dt * acc.x;
            v.y += k.dt * acc.y;
            p.x += k.dt * v.x;
            p.y += k.dt * v.y;
            // tether to the parent (adjustPosition, 1007-1022), parent after its advance
            int parent = H.s_id[i] >> 2;
            int pi = (parent >= 0 && parent < slotsL) ? L.map[parent] : -1;
            if (pi >= 0 && L.s_st[pi] == 1) {
                V2<T> pl = nxt_posL[pi];
                T rho = L.s_dens[pi];
                V2<T> pji{p.x - pl.x, p.y - pl.y};
                T dist = norm2(pji);
                T lim = T(std::fmin(double(dist), 0.75 * std::sqrt(double(k.mL) / (double(rho) * kPi))));
                if (!(k.tether_guard && dist == T(0))) {
                    p.x = pl.x + lim / dist * pji.x;
                    p.y = pl.y + lim / dist * pji.y;
                }
            }
            nxt_posH[i] = p;
            nxt_velH[i] = v;
        }
    }

    int step() {
        const bool carry = k.relax_iters > 0;
        build(H, k.rh, k.dimH, slotsH, carry);
        build(L, k.r, k.dimL, slotsL, carry);
        if (k.relax_iters > 0 && !fresh.empty()) relax();
        density_high();
        density_low();
        force_low();
        force_high();
        // assemble next list-order state
        const int nL = L.n(), nH = H.n();
        const int ns = (int)split.size();
        if (nH + 4 * ns > capH) {
            overflow = 1;
            return TSS_CAPACITY;
        }
        std::vector<int32_t> split_ids(ns);
        for (int q = 0; q < ns; ++q) split_ids[q] = L.s_id[split[q]];
        // low
        L.id = L.s_id;
        L.pos = nxt_posL;
        L.vel = nxt_velL;
        L.st = nxt_stL;
        L.dens = L.s_dens;
        L.pres = L.s_pres;
        // high: existing in sorted order without the children of parents that merged
        // back, then 4 children per split (initSubParticlesAndAddToList)
        std::vector<int32_t> hid;
        std::vector<V2<T>> hpos, hvel;
        std::vector<uint8_t> hst;
        std::vector<T> hd, hp;
        removed = 0;
        for (int i = 0; i < nH; ++i) {
            const int parent = H.s_id[i] >> 2;
            const int pi = (parent >= 0 && parent < slotsL) ? L.map[parent] : -1;
            if (k.merge && pi >= 0 && L.s_st[pi] == 1 && nxt_stL[pi] == 0) {
                ++removed;
                continue;
            }
            hid.push_back(H.s_id[i]);
            hpos.push_back(nxt_posH[i]);
            hvel.push_back(nxt_velH[i]);
            hst.push_back(H.s_st[i]);
            hd.push_back(H.s_dens[i]);
            hp.push_back(H.s_pres[i]);
        }
        for (int q = 0; q < ns; ++q) {
            int i = split[q];
            int id = L.s_id[i];
            V2<T> p = nxt_posL[i], v = nxt_velL[i];
            T rho = L.s_dens[i];
            // the older snapshot's placement: pos +- DIR_LEN*h with h = r, in float
            // (TwoScale2D-master/TwoScale2D/WCSPHSolver.cu:840-850)
            T rad = k.older_place ? T(0.35355339f * float(k.r))
                                  : T(0.5 * std::sqrt(double(k.mL) / (double(T(2) * rho) * kPi)));
            const V2<T> cp[4] = {{p.x + rad, p.y + rad}, {p.x - rad, p.y + rad},
                                 {p.x + rad, p.y - rad}, {p.x - rad, p.y - rad}};
            for (int c = 0; c < 4; ++c) {
                hid.push_back(4 * id + c);
                hpos.push_back(cp[c]);
                hvel.push_back(v);
                hst.push_back(1);
                hd.push_back(T(0));
                hp.push_back(T(0));
            }
        }
        (void)nL;
        H.id.swap(hid);
        H.pos.swap(hpos);
        H.vel.swap(hvel);
        H.st.swap(hst);
        H.dens.swap(hd);
        H.pres.swap(hp);
        fresh = split_ids;
        split = split_ids;
        ++steps_done;
        return TSS_OK;
    }
};

// ---------------------------------------------------------------------------
struct Handle {
    int precision;
    std::unique_ptr<Oracle<float>> f;
    std::unique_ptr<Oracle<double>> d;
};

template <class T>
int set_scale(Oracle<T>& o, int scale, int n, const int32_t* id, const double* pos, const double* vel,
              const uint8_t* st, const double* dens, const double* pres) {
    Scale<T>& S = scale == 0 ? o.L : o.H;
    const int slots = scale == 0 ? o.slotsL : o.slotsH;
    if (n < 0 || (scale == 1 && n > o.capH)) return TSS_INVALID_ARG;
    std::vector<char> seen(slots, 0);
    for (int i = 0; i < n; ++i) {
        if (id[i] < 0 || id[i] >= slots || seen[id[i]]) return TSS_INVALID_ARG;
        seen[id[i]] = 1;
    }
    S.id.assign(id, id + n);
    S.pos.resize(n);
    S.vel.resize(n);
    S.st.assign(st, st + n);
    S.dens.assign(n, T(0));
    S.pres.assign(n, T(0));
    for (int i = 0; i < n; ++i) {
        S.pos[i] = {T(pos[2 * i]), T(pos[2 * i + 1])};
        S.vel[i] = {vel ? T(vel[2 * i]) : T(0), vel ? T(vel[2 * i + 1]) : T(0)};
        if (dens) S.dens[i] = T(dens[i]);
        if (pres) S.pres[i] = T(pres[i]);
    }
    return TSS_OK;
}

template <class T>
int get_buf(Oracle<T>& o, int scale, const char* name, void* dst, size_t cap, size_t* written) {
    Scale<T>& S = scale == 0 ? o.L : o.H;
    std::string nm(name);
    auto put_i = [&](const std::vector<int32_t>& v) {
        if (written) *written = v.size();
        if (dst && cap >= v.size()) std::memcpy(dst, v.data(), v.size() * 4);
        return (dst && cap < v.size()) ? (int)TSS_INVALID_ARG : (int)TSS_OK;
    };
    auto put_u8 = [&](const std::vector<uint8_t>& v) {
        if (written) *written = v.size();
        if (dst && cap >= v.size()) std::memcpy(dst, v.data(), v.size());
        return (dst && cap < v.size()) ? (int)TSS_INVALID_ARG : (int)TSS_OK;
    };
    auto put_s = [&](const std::vector<T>& v) {
        if (written) *written = v.size();
        if (dst && cap < v.size()) return (int)TSS_INVALID_ARG;
        if (dst)
            for (size_t i = 0; i < v.size(); ++i) ((double*)dst)[i] = double(v[i]);
        return (int)TSS_OK;
    };
    auto put_v = [&](const std::vector<V2<T>>& v) {
        if (written) *written = 2 * v.size();
        if (dst && cap < 2 * v.size()) return (int)TSS_INVALID_ARG;
        if (dst)
            for (size_t i = 0; i < v.size(); ++i) {
                ((double*)dst)[2 * i] = double(v[i].x);
                ((double*)dst)[2 * i + 1] = double(v[i].y);
            }
        return (int)TSS_OK;
    };
    if (nm == "id") return put_i(S.id);
    if (nm == "pos") return put_v(S.pos);
    if (nm == "vel") return put_v(S.vel);
    if (nm == "state") return put_u8(S.st);
    if (nm == "dens_state") return put_s(S.dens);
    if (nm == "pres_state") return put_s(S.pres);
    if (nm == "sorted_src") return put_i(S.s_src);
    if (nm == "sorted_id") return put_i(S.s_id);
    if (nm == "cell_off") return put_i(S.off);
    if (nm == "dens") return put_s(S.s_dens);
    if (nm == "pres") return put_s(S.s_pres);
    if (nm == "acc") return put_v(S.s_acc);
    if (nm == "acc_scale") return put_s(S.s_scale);
    if (nm == "split") return put_i(o.split);
    if (nm == "fresh") return put_i(o.fresh);
    if (nm == "wall_cell_off") return put_i(o.wall_off);
    return TSS_INVALID_ARG;
}

}  // namespace

extern "C" {

// Create an oracle; precision 32 (FP32, the reference's arithmetic) or 64.
void* orc_create(const tss_config* cfg, int precision, float mass_low, float mass_high, int n_low_slots,
                 int cap_high, int n_wall, const float* wall_pos, float mass_wall) {
    Handle* h = new Handle();
    h->precision = precision;
    if (precision == 64)
        h->d.reset(new Oracle<double>(*cfg, mass_low, mass_high, mass_wall, n_low_slots, cap_high, n_wall, wall_pos));
    else
        h->f.reset(new Oracle<float>(*cfg, mass_low, mass_high, mass_wall, n_low_slots, cap_high, n_wall, wall_pos));
    return h;
}

void orc_destroy(void* p) { delete (Handle*)p; }

int orc_set_scale(void* p, int scale, int n, const int32_t* id, const double* pos, const double* vel,
                  const uint8_t* st, const double* dens, const double* pres) {
    Handle* h = (Handle*)p;
    return h->f ? set_scale(*h->f, scale, n, id, pos, vel, st, dens, pres)
                : set_scale(*h->d, scale, n, id, pos, vel, st, dens, pres);
}

int orc_set_fresh(void* p, int n, const int32_t* parents) {
    Handle* h = (Handle*)p;
    std::vector<int32_t> v(parents, parents + n);
    if (h->f) h->f->fresh = v; else h->d->fresh = v;
    return TSS_OK;
}

// Headless splat renderer restated on the CPU (the reference's display():
// TwoScale2D/main.cpp:65-102 with QuantityRenderer/PointRenderer and their
// shaders): each particle, in order, blends every pixel whose centre lies in its
// disc; same FP32 expressions as the GPU rasterizer.  view = {xs, ys, xe, ye};
// img holds W*H RGBA floats (row 0 at the bottom) and is blended into.
int orc_splat(const float* view, int W, int H, int n, const float* pos, const float* dens, int nvalid, float rho0,
              const float* rgb, float ps, float* img) {
    const float xs = view[0], ys = view[1], w = view[2] - view[0], h = view[3] - view[1];
    auto clamp01 = [](float v) { return std::fmin(std::fmax(v, 0.0f), 1.0f); };
    for (int i = 0; i < n; ++i) {
        const float cx = (pos[2 * i] - xs) / w * 2.0f - 1.0f;
        const float cy = (pos[2 * i + 1] - ys) / h * 2.0f - 1.0f;
        const float fx0 = (cx - ps + 1.0f) * 0.5f * W - 0.5f, fx1 = (cx + ps + 1.0f) * 0.5f * W - 0.5f;
        const float fy0 = (cy - ps + 1.0f) * 0.5f * H - 0.5f, fy1 = (cy + ps + 1.0f) * 0.5f * H - 0.5f;
        if (!(fx1 >= -1.0f && fx0 <= W && fy1 >= -1.0f && fy0 <= H)) continue;
        const int x0 = std::max(0, (int)std::floor(std::fmax(fx0, -2.0f)) - 1);
        const int x1 = std::min(W - 1, (int)std::ceil(std::fmin(fx1, W + 2.0f)) + 1);
        const int y0 = std::max(0, (int)std::floor(std::fmax(fy0, -2.0f)) - 1);
        const int y1 = std::min(H - 1, (int)std::ceil(std::fmin(fy1, H + 2.0f)) + 1);
        float col[3];
        if (dens) {  // jet colour of min(|rho - rho0|, 400) / 400
            const float rho = i < nvalid ? dens[i] : 0.0f;
            const float f = 4.0f * (std::fmin(std::fabs(rho - rho0), 400.0f) / 400.0f);
            col[0] = clamp01(std::fmin(f - 1.5f, -f + 4.5f));
            col[1] = clamp01(std::fmin(f - 0.5f, -f + 3.5f));
            col[2] = clamp01(std::fmin(f + 0.5f, -f + 2.5f));
        } else {
            col[0] = rgb[0];
            col[1] = rgb[1];
            col[2] = rgb[2];
        }
        for (int py = y0; py <= y1; ++py) {
            const float yp = ((float)py + 0.5f) / (float)H * 2.0f - 1.0f;
            for (int px = x0; px <= x1; ++px) {
                const float xp = ((float)px + 0.5f) / (float)W * 2.0f - 1.0f;
                const float rx = (xp - cx) / ps, ry = (yp - cy) / ps;
                if (rx * rx + ry * ry <= 1.0f) {
                    float* c = img + 4 * ((size_t)py * W + px);
                    c[0] = 0.5f * col[0] + 0.5f * c[0];
                    c[1] = 0.5f * col[1] + 0.5f * c[1];
                    c[2] = 0.5f * col[2] + 0.5f * c[2];
                    c[3] = 0.5f * 0.5f + 0.5f * c[3];
                }
            }
        }
    }
    return TSS_OK;
}

// Steps taken (the moving region of interest's step index), e.g. after loading a
// state taken from a solver after that many steps.
int orc_set_steps(void* p, long long steps) {
    Handle* h = (Handle*)p;
    if (h->f) h->f->steps_done = steps; else h->d->steps_done = steps;
    return TSS_OK;
}

// Whether the next steps also compute each acceleration's error scale ("acc_scale").
int orc_set_want_scale(void* p, int on) {
    Handle* h = (Handle*)p;
    if (h->f) h->f->want_scale = on != 0; else h->d->want_scale = on != 0;
    return TSS_OK;
}

int orc_step(void* p) {
    Handle* h = (Handle*)p;
    return h->f ? h->f->step() : h->d->step();
}

int orc_get(void* p, int scale, const char* name, void* dst, size_t cap, size_t* written) {
    Handle* h = (Handle*)p;
    return h->f ? get_buf(*h->f, scale, name, dst, cap, written) : get_buf(*h->d, scale, name, dst, cap, written);
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Evaluate one kernel function for known-answer tests.  what: 0 = W_s(d),
// 1 = |grad W_s| along +x at distance d, 2 = wall weight Gamma_s(d) with speed of
// sound cs; C and G are derived from r as Bind() does.  precision 32 or 64.
double orc_eval(int what, double d, double r, double cs, int precision) {
    if (precision == 32) {
        float rf = float(r), df = float(d);
        float C = float(20.0 / (14.0 * kPi * double(rf) * double(rf)));
        float G = float(-120.0 / (14.0 * kPi * double(rf) * double(rf) * double(rf)));
        if (what == 0) return W<float>(df, rf, C);
        if (what == 1) return dW<float>({df, 0.f}, df, rf, G).x;
        return gamma_wall<float>(df, rf, float(cs));
    }
    double C = 20.0 / (14.0 * kPi * r * r), G = -120.0 / (14.0 * kPi * r * r * r);
    if (what == 0) return W<double>(d, r, C);
    if (what == 1) return dW<double>({d, 0.0}, d, r, G).x;
    return gamma_wall<double>(d, r, cs);
}

// Grid build alone (FP32): hash, (cell, id) order and dense cell offsets.
int orc_grid(int n, const float* pos, const int32_t* id, float ox, float oy, float cell, int dimx, int dimy,
             int32_t* order, int32_t* cell_off) {
    std::vector<V2<float>> p(n);
    for (int i = 0; i < n; ++i) p[i] = {pos[2 * i], pos[2 * i + 1]};
    int dim[2] = {dimx, dimy};
    std::vector<int32_t> o, off;
    grid_order<float>(n, p.data(), id, ox, oy, cell, dim, o, off);
    std::memcpy(order, o.data(), sizeof(int32_t) * n);
    std::memcpy(cell_off, off.data(), sizeof(int32_t) * off.size());
    return TSS_OK;
}

}  // extern "C"
