// serve.cpp -- the serving loop: continuous batching of scene requests over a pool.
//
// No counterpart in the reference (a desktop program advancing one scene per
// frame, TwoScale2D/main.cpp:65-102).  This is a client of the pool calls of the C
// ABI (include/tss.h):
//
//   * requests become visible at their arrival time and wait in arrival order;
//     the head of the queue is admitted as soon as tss_pool_can_admit says the
//     pool has room (first come, first served: a request that does not fit holds
//     back the ones behind it, so large scenes are not starved)
//   * every admitted scene advances with every other in each step; steps are
//     issued in chunks that end at the next horizon (at most max_steps_per_launch
//     steps), and admission and retirement run between chunks
//   * a scene that reached its horizon is extracted (tss_pool_extract, written by
//     the GPU straight into mapped page-locked memory) and retired; its pages are
//     free for the next admission at once
//   * the host queues at most max_in_flight chunks ahead of the GPU, then waits for
//     the oldest one; its event gives the completion time of the scenes it
//     finished, on the same clock as the arrivals
//
// Uploads go through a page-locked staging ring (so the copies are asynchronous)
// and results come back through a mapped one; both are freed chunk by chunk, in
// order, when the chunk's event has completed.
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/tss.h"

namespace {

size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// FIFO byte ring: allocations are released oldest first.
class ByteRing {
  public:
    bool init(size_t cap, bool mapped) {
        cap_ = al256(cap);
        unsigned flags = mapped ? cudaHostAllocMapped : cudaHostAllocDefault;
        if (cudaHostAlloc(reinterpret_cast<void**>(&host_), cap_, flags) != cudaSuccess) return false;
        dev_ = host_;
        if (mapped) {
            void* d = nullptr;
            if (cudaHostGetDevicePointer(&d, host_, 0) != cudaSuccess) return false;
            dev_ = static_cast<char*>(d);
        }
        return true;
    }
    ~ByteRing() {
        if (host_) cudaFreeHost(host_);
    }
    size_t capacity() const { return cap_; }
    // Offset of n bytes, or false if there is no contiguous room now.  The live
    // allocations occupy [tail, head) or, after a wrap, [tail, end) and [0, head).
    bool alloc(size_t n, size_t* off) {
        n = al256(n > 0 ? n : 1);
        if (n > cap_) return false;
        size_t at;
        if (live_.empty()) {
            at = 0;
        } else if (head_ > tail_) {
            if (cap_ - head_ >= n) at = head_;
            else if (tail_ >= n) at = 0;  // wrap: the end of the buffer stays unused until then
            else return false;
        } else {
            if (tail_ - head_ >= n) at = head_;
            else return false;
        }
        live_.push_back({at, n});
        head_ = at + n;
        tail_ = live_.front().first;
        *off = at;
        return true;
    }
    void release_oldest() {
        if (live_.empty()) return;
        live_.pop_front();
        if (live_.empty()) head_ = tail_ = 0;
        else tail_ = live_.front().first;
    }
    size_t live() const { return live_.size(); }
    char* host(size_t off) const { return host_ + off; }
    char* dev(size_t off) const { return dev_ + off; }

  private:
    char* host_ = nullptr;
    char* dev_ = nullptr;
    size_t cap_ = 0, head_ = 0, tail_ = 0;
    std::deque<std::pair<size_t, size_t>> live_;
};

// Where a finished scene's state sits in the result ring.
struct ResultSlot {
    size_t off = 0;
    int cap[2] = {0, 0};
    size_t a_counts = 0, a_id[2] = {}, a_pos[2] = {}, a_vel[2] = {}, a_st[2] = {}, a_dens[2] = {}, a_pres[2] = {};
};

size_t layout(ResultSlot& r, int n_low) {
    r.cap[0] = n_low;
    r.cap[1] = 4 * n_low;
    size_t o = 0;
    r.a_counts = o;
    o += 256;
    for (int k = 0; k < 2; ++k) {
        const size_t n = static_cast<size_t>(r.cap[k]);
        r.a_id[k] = o;
        o += al256(4 * n);
        r.a_pos[k] = o;
        o += al256(8 * n);
        r.a_vel[k] = o;
        o += al256(8 * n);
        r.a_st[k] = o;
        o += al256(n);
        r.a_dens[k] = o;
        o += al256(4 * n);
        r.a_pres[k] = o;
        o += al256(4 * n);
    }
    return o;
}

struct Active {
    int req;
    int scene;
    int left;
    int64_t first_step;
};

struct Finished {
    int req;
    ResultSlot slot;
};

struct Chunk {
    cudaEvent_t ev = nullptr;
    int n_in = 0, n_out = 0;            // ring allocations owned by this chunk
    std::vector<Finished> done;
};

}  // namespace

struct tss_server {
    tss_server_config cfg{};
    tss_solver* pool = nullptr;
    cudaStream_t stream = nullptr;
    ByteRing in_ring, out_ring;
    std::vector<cudaEvent_t> free_events;
    cudaEvent_t ev0 = nullptr;
    std::string err;

    ~tss_server() {
        if (stream) cudaStreamSynchronize(stream);
        for (cudaEvent_t e : free_events) cudaEventDestroy(e);
        if (ev0) cudaEventDestroy(ev0);
        if (pool) tss_solver_destroy(pool);
        if (stream) cudaStreamDestroy(stream);
    }
    cudaEvent_t event() {
        if (!free_events.empty()) {
            cudaEvent_t e = free_events.back();
            free_events.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreateWithFlags(&e, cudaEventDefault);
        return e;
    }
};

namespace {

using Clock = std::chrono::steady_clock;

struct Run {
    tss_server* sv;
    int n;
    const tss_request* reqs;
    tss_request_stats* stats;
    Clock::time_point t0;
    std::deque<Chunk> inflight;
    Chunk open;                 // allocations and finishers since the last recorded chunk
    int64_t steps = 0;
    double sum_active = 0;
    int max_active = 0;
    int served = 0;
    double last_done = 0;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    // Wait for the oldest chunk: completion times, result copies, ring space.
    tss_status fail(tss_status st, const char* msg) {
        sv->err = msg;
        return st;
    }

    tss_status complete_oldest() {
        Chunk c = std::move(inflight.front());
        inflight.pop_front();
        if (cudaEventSynchronize(c.ev) != cudaSuccess) return fail(TSS_CUDA_ERROR, "waiting for a chunk of steps");
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, sv->ev0, c.ev);
        const double t = ms / 1e3;
        for (const Finished& f : c.done) {
            tss_request_stats& st = stats[f.req];
            const int32_t* cnt = reinterpret_cast<const int32_t*>(sv->out_ring.host(f.slot.off + f.slot.a_counts));
            st.done_s = t;
            st.n_low = cnt[0];
            st.n_high = cnt[1];
            st.status = cnt[2] == 0 ? TSS_OK : TSS_NUMERIC;
            last_done = std::max(last_done, t);
            ++served;
            tss_scene_result* out = reqs[f.req].result;
            if (!out) continue;
            for (int k = 0; k < 2; ++k) {
                const int m = std::min(cnt[k], out->cap[k]);
                out->n[k] = cnt[k];
                const char* b = sv->out_ring.host(f.slot.off);
                if (out->id[k]) std::memcpy(out->id[k], b + f.slot.a_id[k], 4 * static_cast<size_t>(m));
                if (out->pos[k]) std::memcpy(out->pos[k], b + f.slot.a_pos[k], 8 * static_cast<size_t>(m));
                if (out->vel[k]) std::memcpy(out->vel[k], b + f.slot.a_vel[k], 8 * static_cast<size_t>(m));
                if (out->state[k]) std::memcpy(out->state[k], b + f.slot.a_st[k], static_cast<size_t>(m));
                if (out->dens[k]) std::memcpy(out->dens[k], b + f.slot.a_dens[k], 4 * static_cast<size_t>(m));
                if (out->pres[k]) std::memcpy(out->pres[k], b + f.slot.a_pres[k], 4 * static_cast<size_t>(m));
            }
        }
        for (int k = 0; k < c.n_in; ++k) sv->in_ring.release_oldest();
        for (int k = 0; k < c.n_out; ++k) sv->out_ring.release_oldest();
        sv->free_events.push_back(c.ev);
        return TSS_OK;
    }

    tss_status record_open() {
        open.ev = sv->event();
        if (!open.ev || cudaEventRecord(open.ev, sv->stream) != cudaSuccess)
            return fail(TSS_CUDA_ERROR, "recording a chunk's event");
        inflight.push_back(std::move(open));
        open = Chunk{};
        return TSS_OK;
    }

    tss_status drain() {
        while (!inflight.empty())
            if (tss_status st = complete_oldest(); st != TSS_OK) return st;
        return TSS_OK;
    }

    // Try to admit request r: TSS_OK, TSS_CAPACITY (not now) or TSS_INVALID_ARG (never).
    tss_status try_admit(int r, std::vector<Active>& active) {
        const tss_scene_desc& d = reqs[r].scene;
        tss_status chk = tss_pool_can_admit(sv->pool, &d);
        if (chk != TSS_OK) return chk;
        const size_t nb = 8 * static_cast<size_t>(d.n_low), wb = 8 * static_cast<size_t>(d.n_wall);
        const size_t need = al256(nb) * (d.low_vel ? 2 : 1) + al256(wb);
        if (need > sv->in_ring.capacity()) return TSS_INVALID_ARG;
        size_t off = 0;
        if (!sv->in_ring.alloc(need, &off)) return TSS_CAPACITY;
        ++open.n_in;
        char* h = sv->in_ring.host(off);
        tss_scene_desc s = d;
        std::memcpy(h, d.low_pos, nb);
        s.low_pos = reinterpret_cast<const float*>(h);
        size_t o = al256(nb);
        if (d.low_vel) {
            std::memcpy(h + o, d.low_vel, nb);
            s.low_vel = reinterpret_cast<const float*>(h + o);
            o += al256(nb);
        }
        if (d.n_wall > 0) {
            std::memcpy(h + o, d.wall_pos, wb);
            s.wall_pos = reinterpret_cast<const float*>(h + o);
        }
        int id = -1;
        tss_status st = tss_pool_admit(sv->pool, &s, sv->stream, &id);
        if (st != TSS_OK) return fail(st == TSS_CAPACITY ? TSS_CUDA_ERROR : st, "admission failed after the pool reported room");
        active.push_back({r, id, reqs[r].horizon, steps});
        stats[r].admit_s = now();
        stats[r].first_step = steps;
        return TSS_OK;
    }

    // Extract and retire a scene that reached its horizon.
    tss_status finish(const Active& a) {
        const int n_low = reqs[a.req].scene.n_low;
        ResultSlot slot;
        const size_t need = layout(slot, n_low);
        if (need > sv->out_ring.capacity()) {
            stats[a.req].status = TSS_CAPACITY;  // result larger than the staging ring
            return tss_pool_retire(sv->pool, a.scene, sv->stream);
        }
        size_t off = 0;
        while (!sv->out_ring.alloc(need, &off)) {
            if (!open.done.empty() || open.n_in || open.n_out) {
                if (tss_status st = record_open(); st != TSS_OK) return st;
            }
            if (inflight.empty()) return fail(TSS_CAPACITY, "no room for a result in the empty result ring");
            if (tss_status st = complete_oldest(); st != TSS_OK) return st;
        }
        ++open.n_out;
        slot.off = off;
        char* d = sv->out_ring.dev(off);
        tss_scene_result r{};
        for (int k = 0; k < 2; ++k) {
            r.cap[k] = slot.cap[k];
            r.id[k] = reinterpret_cast<int32_t*>(d + slot.a_id[k]);
            r.pos[k] = reinterpret_cast<float*>(d + slot.a_pos[k]);
            r.vel[k] = reinterpret_cast<float*>(d + slot.a_vel[k]);
            r.state[k] = reinterpret_cast<uint8_t*>(d + slot.a_st[k]);
            r.dens[k] = reinterpret_cast<float*>(d + slot.a_dens[k]);
            r.pres[k] = reinterpret_cast<float*>(d + slot.a_pres[k]);
        }
        tss_status st = tss_pool_extract(sv->pool, a.scene, &r, reinterpret_cast<int32_t*>(d + slot.a_counts), sv->stream);
        if (st != TSS_OK) return st;
        if ((st = tss_pool_retire(sv->pool, a.scene, sv->stream)) != TSS_OK) return st;
        open.done.push_back({a.req, slot});
        return TSS_OK;
    }
};

}  // namespace

extern "C" {

tss_status tss_server_set_arith(tss_server* sv, int mode) {
    if (!sv) return TSS_INVALID_ARG;
    return tss_solver_set_arith(sv->pool, mode);
}

tss_status tss_server_create(const tss_server_config* cfg, tss_server** out) {
    if (!cfg || !out || cfg->max_steps_per_launch < 1 || cfg->max_in_flight < 1 || cfg->staging_bytes < (1 << 20))
        return TSS_INVALID_ARG;
    *out = nullptr;
    tss_server* sv = new (std::nothrow) tss_server();
    if (!sv) return TSS_OOM;
    sv->cfg = *cfg;
    tss_status st = tss_pool_create(&cfg->pool, &sv->pool);
    if (st != TSS_OK) {
        delete sv;
        return st;
    }
    const size_t half = static_cast<size_t>(cfg->staging_bytes) / 2;
    if (cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&sv->ev0) != cudaSuccess || !sv->in_ring.init(half, false) || !sv->out_ring.init(half, true)) {
        delete sv;
        return TSS_CUDA_ERROR;
    }
    *out = sv;
    return TSS_OK;
}

void tss_server_destroy(tss_server* sv) { delete sv; }

tss_status tss_server_last_error(tss_server* sv, char* buf, int len) {
    if (!sv || !buf || len <= 0) return TSS_INVALID_ARG;
    std::string msg = sv->err;
    if (msg.empty() && sv->pool) {  // a pool call's own message
        char pbuf[512];
        if (tss_solver_last_error(sv->pool, pbuf, sizeof pbuf) == TSS_OK) msg = pbuf;
    }
    std::snprintf(buf, static_cast<size_t>(len), "%s", msg.c_str());
    return TSS_OK;
}

tss_status tss_server_run(tss_server* sv, int n, const tss_request* reqs, tss_request_stats* stats,
                          tss_serve_summary* summary) {
    if (!sv || n < 0 || (n > 0 && (!reqs || !stats))) return TSS_INVALID_ARG;
    sv->err.clear();
    for (int i = 0; i < n; ++i)
        if (reqs[i].horizon < 1 || !(reqs[i].arrival_s >= 0.0)) return TSS_INVALID_ARG;
    std::vector<int> order(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return reqs[a].arrival_s < reqs[b].arrival_s; });
    for (int i = 0; i < n; ++i) {
        stats[i] = tss_request_stats{};
        stats[i].arrival_s = reqs[i].arrival_s;
        stats[i].admit_s = stats[i].done_s = -1.0;
        stats[i].first_step = -1;
        stats[i].status = TSS_CUDA_ERROR;  // not served: the run stopped before it (replaced below)
    }
    Run R{sv, n, reqs, stats, {}};
    // the GPU clock and the host clock start together
    if (cudaEventRecord(sv->ev0, sv->stream) != cudaSuccess || cudaEventSynchronize(sv->ev0) != cudaSuccess)
        return TSS_CUDA_ERROR;
    R.t0 = Clock::now();
    size_t next = 0;
    std::deque<int> queue;
    std::vector<Active> active;
    const int kmax = sv->cfg.max_steps_per_launch;
    tss_status st = TSS_OK;
    for (;;) {
        const double t = R.now();
        while (next < order.size() && reqs[order[next]].arrival_s <= t) queue.push_back(order[next++]);
        // admissions, first come first served
        while (!queue.empty()) {
            const int r = queue.front();
            const tss_status a = R.try_admit(r, active);
            if (a == TSS_OK) {
                queue.pop_front();
            } else if (a == TSS_CAPACITY) {
                break;
            } else if (a == TSS_INVALID_ARG) {  // can never fit: rejected
                stats[r].status = TSS_INVALID_ARG;
                queue.pop_front();
            } else {
                st = a;
                break;
            }
        }
        if (st != TSS_OK) break;
        if (active.empty()) {
            if (R.open.n_in || R.open.n_out || !R.open.done.empty()) {
                if ((st = R.record_open()) != TSS_OK) break;
            }
            if (!R.inflight.empty()) {
                if ((st = R.complete_oldest()) != TSS_OK) break;
                continue;
            }
            if (next >= order.size() && queue.empty()) break;
            if (!queue.empty()) {  // nothing runs and the head still does not fit: it never will
                stats[queue.front()].status = TSS_INVALID_ARG;
                queue.pop_front();
                continue;
            }
            const double wait = reqs[order[next]].arrival_s - R.now();
            if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(wait));
            continue;
        }
        int k = kmax;
        for (const Active& a : active) k = std::min(k, a.left);
        if ((st = tss_solver_step(sv->pool, k, sv->stream)) != TSS_OK) break;
        R.steps += k;
        R.sum_active += static_cast<double>(k) * active.size();
        R.max_active = std::max(R.max_active, static_cast<int>(active.size()));
        std::vector<Active> still;
        still.reserve(active.size());
        for (Active& a : active) {
            a.left -= k;
            if (a.left > 0) {
                still.push_back(a);
            } else if ((st = R.finish(a)) != TSS_OK) {
                break;
            }
        }
        if (st != TSS_OK) break;
        active.swap(still);
        if ((st = R.record_open()) != TSS_OK) break;
        while (static_cast<int>(R.inflight.size()) > sv->cfg.max_in_flight)
            if ((st = R.complete_oldest()) != TSS_OK) break;
        if (st != TSS_OK) break;
    }
    if (st == TSS_OK) st = R.drain();
    if (st == TSS_OK) {
        // a scene that went unstable is that request's failure (TSS_NUMERIC in its
        // stats); any other device error fails the run
        st = tss_solver_sync(sv->pool);
        if (st == TSS_NUMERIC) st = TSS_OK;
    }
    if (summary) {
        summary->makespan_s = R.last_done;
        summary->steps = R.steps;
        int64_t ss = 0;
        double ps = 0;
        for (int i = 0; i < n; ++i)
            if (stats[i].status == TSS_OK || stats[i].status == TSS_NUMERIC) {
                ss += reqs[i].horizon;
                ps += static_cast<double>(reqs[i].scene.n_low) * reqs[i].horizon;
            }
        summary->scene_steps = ss;
        summary->low_particle_steps = ps;
        summary->mean_active = R.steps ? R.sum_active / static_cast<double>(R.steps) : 0.0;
        summary->max_active = R.max_active;
        summary->served = R.served;
    }
    return st;
}

}  // extern "C"
