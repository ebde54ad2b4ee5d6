// server.cu -- serving runtime for many SLAM sessions on one GPU.
//
// The reference tracks one map, one frame at a time, under a global mutex
// (GSSlam's optimization_mutex_, src/GSSlam.cu:826,984).  Here any number of
// sessions (each its own map, frame size and pose state, all resident in HBM)
// share the GPU:
//  * admission: a session is admitted while the footprints of the admitted
//    sessions fit the memory budget; otherwise its admission is refused and
//    the caller retries once others have been released;
//  * continuous batching: requests are queued per session (a session's frames
//    depend on each other and run in order); a worker thread launches the
//    next request of every idle admitted session as soon as a slot is free
//    (at most max_inflight frames on the device), so frames of different
//    sessions overlap on the GPU, each on its session's stream, each from
//    the session's captured frame graph; completed frames are collected by
//    polling their events, without blocking on any one of them;
//  * every result carries its arrival, launch and completion times, from
//    which the caller computes latency percentiles.
// A session's results are the same alone and in the mix: its kernels read
// and write only its own buffers, in the same order, with the same launch
// shapes.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/fvgs.h"
#include "../../include/fvgs_server.h"

namespace {

double now_s() {
    using clock = std::chrono::steady_clock;
    return std::chrono::duration<double>(clock::now().time_since_epoch()).count();
}

struct Slot {
    fvgs_session* session = nullptr;
    uint64_t footprint = 0;
    bool active = false;
    bool busy = false;  // a frame of this session is on the device
    std::deque<fvgs_server_request> queue;
    fvgs_server_request running{};
    double t_launch = 0.0;
};

}  // namespace

struct fvgs_server {
    uint64_t budget = 0;
    uint64_t admitted_bytes = 0;
    int max_inflight = 1;
    int inflight = 0;
    std::deque<Slot> slots;  // references stay valid when sessions are added
    std::deque<fvgs_server_result> done;
    std::mutex mu;
    std::condition_variable cv;
    std::atomic<bool> stop{false};
    std::thread worker;
    uint64_t launched = 0, completed = 0;

    void run() {
        std::vector<std::pair<int, Slot*>> to_poll;  // element addresses of a deque stay valid
        while (!stop.load()) {
            bool did_work = false;
            {
                std::unique_lock<std::mutex> lk(mu);
                // launch: idle sessions with queued requests, while slots last
                for (size_t i = 0; i < slots.size() && inflight < max_inflight; ++i) {
                    Slot& sl = slots[i];
                    if (!sl.active || sl.busy || sl.queue.empty()) continue;
                    sl.running = sl.queue.front();
                    sl.queue.pop_front();
                    const fvgs_server_request& r = sl.running;
                    int rc = FVGS_OK;
                    if (r.pyr_levels > 0 && r.pyr_frames) {
                        int w = r.width, h = r.height;
                        const float* p = r.pyr_frames;
                        for (int l = 0; l < r.pyr_levels && rc == FVGS_OK; ++l) {
                            const size_t px = (size_t)w * h;
                            rc = fvgs_set_frame(sl.session, l, p, p + 3 * px, p + 4 * px, p + 7 * px, w, h);
                            p += 10 * px;
                            w = (w + 1) / 2;
                            h = (h + 1) / 2;
                        }
                    } else if (r.rgb)
                        rc = fvgs_set_frame(sl.session, r.level, r.rgb, r.depth, r.grad_x, r.grad_y, r.width,
                                            r.height);
                    else if (r.raw_color)
                        rc = fvgs_preprocess_frame(sl.session, r.raw_color, r.raw_depth, r.raw_depth_u16_mm, r.width,
                                                   r.height, r.raw_levels > 0 ? r.raw_levels : 1, r.raw_double_scale);
                    if (rc == FVGS_OK)
                        rc = r.pyr_levels > 0
                                 ? fvgs_frame_submit_pyramid(sl.session, &r.pose, &r.K, r.pyr_iterations,
                                                             r.pyr_levels, r.map_eta)
                                 : fvgs_frame_submit(sl.session, &r.pose, &r.K, r.level, r.iterations, r.map_eta);
                    sl.t_launch = now_s();
                    if (rc != FVGS_OK) {
                        fvgs_server_result res{};
                        res.tag = r.tag;
                        res.slot = (int)i;
                        res.status = rc;
                        res.pose = r.pose;
                        res.t_arrival = r.t_arrival;
                        res.t_launch = sl.t_launch;
                        res.t_done = sl.t_launch;
                        done.push_back(res);
                        ++completed;
                        continue;
                    }
                    sl.busy = true;
                    ++inflight;
                    ++launched;
                    did_work = true;
                }
                to_poll.clear();
                for (size_t i = 0; i < slots.size(); ++i)
                    if (slots[i].busy) to_poll.emplace_back((int)i, &slots[i]);
            }
            // collect finished frames (the sessions involved are only touched
            // by this thread while busy)
            for (const auto& entry : to_poll) {
                const int i = entry.first;
                Slot& sl = *entry.second;
                int finished = 0;
                int rc = fvgs_frame_poll(sl.session, &finished);
                if (rc == FVGS_OK && !finished) continue;
                fvgs_server_result res{};
                res.tag = sl.running.tag;
                res.slot = i;
                res.pose = sl.running.pose;
                if (rc == FVGS_OK) rc = fvgs_frame_wait(sl.session, &res.pose, res.last_step);
                res.status = rc;
                res.t_arrival = sl.running.t_arrival;
                res.t_launch = sl.t_launch;
                res.t_done = now_s();
                std::lock_guard<std::mutex> lk(mu);
                sl.busy = false;
                --inflight;
                ++completed;
                done.push_back(res);
                did_work = true;
            }
            if (did_work) {
                cv.notify_all();
            } else {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait_for(lk, std::chrono::microseconds(to_poll.empty() ? 500 : 20));
            }
        }
    }
};

extern "C" {

int fvgs_server_create(uint64_t memory_budget_bytes, int max_inflight, fvgs_server** out) {
    if (!out || max_inflight <= 0) return FVGS_E_INVALID;
    *out = nullptr;
    fvgs_server* sv = new (std::nothrow) fvgs_server();
    if (!sv) return FVGS_E_NOMEM;
    sv->budget = memory_budget_bytes;
    sv->max_inflight = max_inflight;
    try {
        sv->worker = std::thread([sv] { sv->run(); });
    } catch (...) {
        delete sv;
        return FVGS_E_NOMEM;
    }
    *out = sv;
    return FVGS_OK;
}

int fvgs_server_destroy(fvgs_server* sv) {
    if (!sv) return FVGS_E_INVALID;
    // let the frames on the device finish, then stop the worker
    for (;;) {
        std::unique_lock<std::mutex> lk(sv->mu);
        bool pending = sv->inflight > 0;
        for (auto& sl : sv->slots) pending = pending || (sl.active && !sl.queue.empty());
        if (!pending) break;
        sv->cv.wait_for(lk, std::chrono::milliseconds(1));
    }
    sv->stop.store(true);
    sv->cv.notify_all();
    if (sv->worker.joinable()) sv->worker.join();
    delete sv;
    return FVGS_OK;
}

int fvgs_server_admit(fvgs_server* sv, fvgs_session* s, int* slot) {
    if (!sv || !s || !slot) return FVGS_E_INVALID;
    uint64_t fp = 0;
    const int rc = fvgs_session_footprint(s, &fp);
    if (rc != FVGS_OK) return rc;
    std::lock_guard<std::mutex> lk(sv->mu);
    for (auto& sl : sv->slots)
        if (sl.active && sl.session == s) return FVGS_E_STATE;
    if (sv->admitted_bytes + fp > sv->budget) return FVGS_E_ADMISSION;
    int idx = -1;
    for (size_t i = 0; i < sv->slots.size(); ++i)
        if (!sv->slots[i].active) {
            idx = (int)i;
            break;
        }
    if (idx < 0) {
        sv->slots.emplace_back();
        idx = (int)sv->slots.size() - 1;
    }
    Slot& sl = sv->slots[idx];
    sl = Slot();
    sl.session = s;
    sl.footprint = fp;
    sl.active = true;
    sv->admitted_bytes += fp;
    *slot = idx;
    return FVGS_OK;
}

int fvgs_server_release(fvgs_server* sv, int slot) {
    if (!sv) return FVGS_E_INVALID;
    std::unique_lock<std::mutex> lk(sv->mu);
    if (slot < 0 || slot >= (int)sv->slots.size() || !sv->slots[slot].active) return FVGS_E_INVALID;
    // wait for the session's queued and running frames
    while (sv->slots[slot].busy || !sv->slots[slot].queue.empty()) sv->cv.wait_for(lk, std::chrono::milliseconds(1));
    sv->admitted_bytes -= sv->slots[slot].footprint;
    sv->slots[slot] = Slot();
    return FVGS_OK;
}

int fvgs_server_submit(fvgs_server* sv, int slot, const fvgs_server_request* req) {
    if (!sv || !req) return FVGS_E_INVALID;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (slot < 0 || slot >= (int)sv->slots.size() || !sv->slots[slot].active) return FVGS_E_INVALID;
    fvgs_server_request r = *req;
    if (r.t_arrival <= 0.0) r.t_arrival = now_s();
    sv->slots[slot].queue.push_back(r);
    sv->cv.notify_all();
    return FVGS_OK;
}

int fvgs_server_results(fvgs_server* sv, fvgs_server_result* out, int max_results, int wait_for, int* n) {
    if (!sv || !n || max_results < 0 || (max_results > 0 && !out)) return FVGS_E_INVALID;
    std::unique_lock<std::mutex> lk(sv->mu);
    while ((int)sv->done.size() < wait_for && !sv->stop.load()) {
        bool possible = sv->inflight > 0;
        for (auto& sl : sv->slots) possible = possible || (sl.active && !sl.queue.empty());
        if (!possible) break;  // nothing left that could complete
        sv->cv.wait_for(lk, std::chrono::milliseconds(1));
    }
    int k = 0;
    while (k < max_results && !sv->done.empty()) {
        out[k++] = sv->done.front();
        sv->done.pop_front();
    }
    *n = k;
    return FVGS_OK;
}

int fvgs_server_now(double* seconds) {
    if (!seconds) return FVGS_E_INVALID;
    *seconds = now_s();
    return FVGS_OK;
}

int fvgs_server_stats(fvgs_server* sv, uint64_t* admitted_bytes, int* inflight, uint64_t* launched,
                      uint64_t* completed) {
    if (!sv) return FVGS_E_INVALID;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (admitted_bytes) *admitted_bytes = sv->admitted_bytes;
    if (inflight) *inflight = sv->inflight;
    if (launched) *launched = sv->launched;
    if (completed) *completed = sv->completed;
    return FVGS_OK;
}

}  // extern "C"
