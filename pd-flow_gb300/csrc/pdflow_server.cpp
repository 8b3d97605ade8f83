// Request loop for many camera streams (include/pdflow_server.h).
//
// Threads: the caller's threads submit and wait; one worker per lane forms
// and runs batches.  One mutex guards the request table, the lanes' pending
// queues and the stream table; solves run outside it.  Each lane owns its
// solver handle (and its own network instance for the learned path), so
// lanes never share device buffers and run concurrently.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <queue>
#include <random>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/pdflow.h"
#include "../../include/pdflow_net.h"
#include "../../include/pdflow_server.h"
#include "pdflow_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    unsigned long long id = 0;
    unsigned stream = 0, slot = 0;
    unsigned long long frame = 0;
    std::vector<uint8_t> inten;
    std::vector<uint16_t> depth;
    Clock::time_point t_submit, t_start, t_done;
    int status = PDFLOW_OK;
    bool has_flow = false;
    bool done = false;
    unsigned batch_pairs = 0, batch_fallbacks = 0;
    std::vector<float> dx, dy, dz;
};

struct Lane {
    unsigned width = 0, height = 0, rows = 0, cols = 0;
    pdflow_solver* solver = nullptr;
    pdflow_net* net = nullptr;
    std::vector<int> slot_stream;           // stream id per slot, -1 = free
    std::deque<Request*> pending;
    std::condition_variable cv;             // the lane's worker waits here for pending frames
    std::thread worker;
    uint8_t* st_i = nullptr;                // pinned staging [slots][h][w]
    uint16_t* st_z = nullptr;
    float* out = nullptr;                   // pinned flows [3][slots][rows*cols]
    size_t device_bytes = 0;
};

struct Stream {
    bool open = false;
    unsigned lane = 0, slot = 0;
    unsigned long long frames = 0;          // submitted
    unsigned inflight = 0;
};

}  // namespace

struct pdflow_server {
    pdflow_server_config cfg{};
    std::vector<float> params;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_done;
    int device = 0;
    std::vector<std::unique_ptr<Lane>> lanes;
    std::vector<Stream> streams;
    std::unordered_map<unsigned long long, Request*> requests;
    unsigned long long next_id = 1;
    bool stop = false;
    size_t device_bytes = 0;
    pdflow_server_stats stats{};
};

namespace {

double ms_since(const pdflow_server* s, Clock::time_point t)
{
    return std::chrono::duration<double, std::milli>(t - s->t0).count();
}

int fail(int code, const char* what)
{
    pdflow::set_last_error(what);
    return code;
}

void destroy_lane(Lane* L)
{
    if (L->solver) pdflow_destroy(L->solver);
    if (L->net) pdflow_net_destroy(L->net);
    if (L->st_i) cudaFreeHost(L->st_i);
    if (L->st_z) cudaFreeHost(L->st_z);
    if (L->out) cudaFreeHost(L->out);
}

// Runs one batch of a lane (outside the server lock).
void run_batch(pdflow_server* srv, Lane* L, std::vector<Request*>& batch)
{
    const pdflow::NvtxRange trace_range("server lane batch");
    const unsigned n = unsigned(batch.size());
    const size_t img = size_t(L->width) * L->height;
    const size_t N = size_t(L->rows) * L->cols;
    std::vector<unsigned> slots(n), solve_slots;
    std::vector<unsigned> solve_idx;
    for (unsigned k = 0; k < n; ++k) {
        Request* r = batch[k];
        slots[k] = r->slot;
        std::memcpy(L->st_i + k * img, r->inten.data(), img);
        std::memcpy(L->st_z + k * img, r->depth.data(), img * 2);
        if (r->frame > 0) {
            solve_slots.push_back(slots[k]);
            solve_idx.push_back(k);
        }
    }
    int rc = pdflow_push_frames_slots_u16(L->solver, n, slots.data(), L->st_i, L->st_z);
    pdflow_learned_report rep{0, 0.f};
    const unsigned m = unsigned(solve_slots.size());
    if (rc == PDFLOW_OK && m > 0) {
        if (srv->cfg.learned) {
            pdflow_learned_opts o{srv->cfg.iter_scale, srv->cfg.energy_margin};
            rc = pdflow_solve_slots_learned(L->solver, m, solve_slots.data(), L->net, &o, &rep);
        } else {
            rc = pdflow_solve_slots(L->solver, m, solve_slots.data());
        }
        if (rc == PDFLOW_OK)
            rc = pdflow_read_flow_slots(L->solver, m, solve_slots.data(), L->out, L->out + size_t(m) * N,
                                        L->out + size_t(2) * m * N);
    } else if (rc == PDFLOW_OK) {
        rc = pdflow_synchronize(L->solver);
    }
    const auto t_done = Clock::now();
    // results into the requests and their frames freed before the server's
    // lock: nothing else touches a request of this batch until it is done
    for (unsigned j = 0; j < m && rc == PDFLOW_OK; ++j) {
        Request* r = batch[solve_idx[j]];
        r->dx.assign(L->out + j * N, L->out + (j + 1) * N);
        r->dy.assign(L->out + (m + j) * N, L->out + (m + j + 1) * N);
        r->dz.assign(L->out + (2 * m + j) * N, L->out + (2 * m + j + 1) * N);
        r->has_flow = true;
    }
    for (Request* r : batch) {
        r->inten.clear();
        r->inten.shrink_to_fit();
        r->depth.clear();
        r->depth.shrink_to_fit();
    }
    std::lock_guard<std::mutex> lk(srv->mu);
    for (Request* r : batch) {
        r->status = rc;
        r->done = true;
        r->t_done = t_done;
        r->batch_pairs = m;
        r->batch_fallbacks = rep.fallbacks;
        srv->streams[r->stream].inflight--;
    }
    srv->stats.completed += n;
    srv->stats.batches += 1;
    srv->stats.pairs_solved += m;
    srv->stats.fallbacks += rep.fallbacks;
    srv->cv_done.notify_all();
}

void lane_worker(pdflow_server* srv, Lane* L)
{
    cudaSetDevice(srv->device);
    for (;;) {
        std::vector<Request*> batch;
        {
            std::unique_lock<std::mutex> lk(srv->mu);
            L->cv.wait(lk, [&] { return srv->stop || !L->pending.empty(); });
            if (L->pending.empty()) return;   // stop requested and nothing left
            // the oldest pending frame of each stream, in arrival order
            std::vector<unsigned char> taken(srv->streams.size(), 0);
            for (auto it = L->pending.begin(); it != L->pending.end();) {
                Request* r = *it;
                if (!taken[r->stream]) {
                    taken[r->stream] = 1;
                    r->t_start = Clock::now();
                    batch.push_back(r);
                    it = L->pending.erase(it);
                } else {
                    ++it;
                }
            }
        }
        run_batch(srv, L, batch);
    }
}

// Creates a lane for width x height frames if the budget allows.
int add_lane(pdflow_server* srv, unsigned width, unsigned height, Lane** out)
{
    auto L = std::make_unique<Lane>();
    L->width = width;
    L->height = height;
    L->rows = height;
    L->cols = height * 4 / 3;
    const unsigned S = srv->cfg.slots_per_lane;
    int rc = pdflow_create_batch(L->rows, width, height, nullptr, S, &L->solver);
    if (rc) return rc;
    L->device_bytes = pdflow_device_bytes(L->solver);
    if (srv->cfg.learned) {
        L->device_bytes += pdflow::learned_keep_bytes(S);   // allocated by the first learned solve
        rc = pdflow_net_create(S, 1, &L->net);
        if (!rc) rc = pdflow_net_set_params(L->net, srv->params.data(), srv->params.size());
        if (rc) {
            destroy_lane(L.get());
            return rc;
        }
        L->device_bytes += pdflow_net_device_bytes(L->net);
    }
    if (srv->device_bytes + L->device_bytes > srv->cfg.device_budget_bytes) {
        destroy_lane(L.get());
        return fail(PDFLOW_ERR_OOM, "admission refused: a new lane would exceed the device budget");
    }
    const size_t img = size_t(width) * height;
    cudaError_t e = cudaMallocHost(&L->st_i, img * S);
    if (e == cudaSuccess) e = cudaMallocHost(&L->st_z, img * S * 2);
    if (e == cudaSuccess) e = cudaMallocHost(&L->out, sizeof(float) * 3 * S * size_t(L->rows) * L->cols);
    if (e != cudaSuccess) {
        destroy_lane(L.get());
        return pdflow::set_error_code(PDFLOW_ERR_OOM, "pinned staging", e);
    }
    L->slot_stream.assign(S, -1);
    // Warm-up: capture the lane's solve graphs for every batch size now, on
    // blank frames, so no live request pays for a graph capture.
    {
        std::memset(L->st_i, 0, img * S);
        std::memset(L->st_z, 0, img * S * 2);
        std::vector<unsigned> slots(S);
        for (unsigned k = 0; k < S; ++k) slots[k] = k;
        rc = pdflow_push_frames_slots_u16(L->solver, S, slots.data(), L->st_i, L->st_z);
        if (!rc) rc = pdflow_push_frames_slots_u16(L->solver, S, slots.data(), L->st_i, L->st_z);
        for (unsigned n = 1; n <= S && !rc; ++n) {
            if (srv->cfg.learned) {
                pdflow_learned_opts o{srv->cfg.iter_scale, srv->cfg.energy_margin};
                rc = pdflow_solve_slots_learned(L->solver, n, slots.data(), L->net, &o, nullptr);
            } else {
                rc = pdflow_solve_slots(L->solver, n, slots.data());
            }
            // and the learned solve's fallback continuation for n pairs
            if (!rc && srv->cfg.learned) {
                pdflow_learned_opts o{srv->cfg.iter_scale, srv->cfg.energy_margin};
                rc = pdflow::learned_solve_all_fallback(L->solver, n, slots.data(), L->net, &o);
            }
        }
        if (!rc) rc = pdflow_synchronize(L->solver);
        if (rc) {
            destroy_lane(L.get());
            return rc;
        }
    }
    srv->device_bytes += L->device_bytes;
    Lane* raw = L.get();
    srv->lanes.push_back(std::move(L));
    raw->worker = std::thread(lane_worker, srv, raw);
    *out = raw;
    return PDFLOW_OK;
}

}  // namespace

extern "C" {

int pdflow_server_create(const pdflow_server_config* cfg, pdflow_server** out)
{
    if (!cfg || !out) return fail(PDFLOW_ERR_ARG, "null argument");
    *out = nullptr;
    if (cfg->slots_per_lane == 0 || cfg->slots_per_lane > 64) return fail(PDFLOW_ERR_ARG, "slots_per_lane: 1..64");
    if (cfg->learned) {
        if (!cfg->net_params || cfg->net_param_count == 0) return fail(PDFLOW_ERR_ARG, "learned needs net_params");
        if (!(cfg->iter_scale > 0.f) || cfg->iter_scale > 1.f) return fail(PDFLOW_ERR_ARG, "iter_scale in (0, 1]");
    }
    pdflow_server* s = new (std::nothrow) pdflow_server();
    if (!s) return fail(PDFLOW_ERR_OOM, "host allocation");
    s->cfg = *cfg;
    if (cfg->learned) s->params.assign(cfg->net_params, cfg->net_params + cfg->net_param_count);
    s->cfg.net_params = nullptr;
    s->t0 = Clock::now();
    cudaGetDevice(&s->device);
    *out = s;
    return PDFLOW_OK;
}

int pdflow_server_destroy(pdflow_server* s)
{
    if (!s) return PDFLOW_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    for (auto& L : s->lanes) L->cv.notify_all();
    for (auto& L : s->lanes)
        if (L->worker.joinable()) L->worker.join();
    for (auto& L : s->lanes) destroy_lane(L.get());
    for (auto& kv : s->requests) delete kv.second;
    delete s;
    return PDFLOW_OK;
}

int pdflow_server_open_stream(pdflow_server* s, unsigned width, unsigned height, unsigned* stream_id)
{
    if (!s || !stream_id) return fail(PDFLOW_ERR_ARG, "null argument");
    if (!((width == 640 && height == 480) || (width == 320 && height == 240)))
        return fail(PDFLOW_ERR_ARG, "frames must be 640x480 or 320x240");
    std::lock_guard<std::mutex> lk(s->mu);
    Lane* lane = nullptr;
    unsigned li = 0, slot = 0;
    for (unsigned i = 0; i < s->lanes.size() && !lane; ++i) {
        Lane* L = s->lanes[i].get();
        if (L->width != width || L->height != height) continue;
        for (unsigned k = 0; k < L->slot_stream.size(); ++k)
            if (L->slot_stream[k] < 0) {
                lane = L;
                li = i;
                slot = k;
                break;
            }
    }
    if (!lane) {
        int rc = add_lane(s, width, height, &lane);
        if (rc) return rc;
        li = unsigned(s->lanes.size() - 1);
        slot = 0;
    }
    unsigned id = 0;
    while (id < s->streams.size() && s->streams[id].open) ++id;
    if (id == s->streams.size()) s->streams.push_back(Stream{});
    Stream& st = s->streams[id];
    st = Stream{};
    st.open = true;
    st.lane = li;
    st.slot = slot;
    lane->slot_stream[slot] = int(id);
    s->stats.streams++;
    *stream_id = id;
    return PDFLOW_OK;
}

int pdflow_server_close_stream(pdflow_server* s, unsigned id)
{
    if (!s) return fail(PDFLOW_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (id >= s->streams.size() || !s->streams[id].open) return fail(PDFLOW_ERR_ARG, "no such stream");
    if (s->streams[id].inflight) return fail(PDFLOW_ERR_STATE, "the stream has frames in flight");
    Stream& st = s->streams[id];
    s->lanes[st.lane]->slot_stream[st.slot] = -1;
    st.open = false;
    s->stats.streams--;
    return PDFLOW_OK;
}

int pdflow_server_submit(pdflow_server* s, unsigned id, const uint8_t* intensity, const uint16_t* depth,
                         unsigned long long* request_id)
{
    if (!s || !intensity || !depth) return fail(PDFLOW_ERR_ARG, "null argument");
    Request* r = new (std::nothrow) Request();
    if (!r) return fail(PDFLOW_ERR_OOM, "host allocation");
    r->t_submit = Clock::now();
    size_t img = 0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (id < s->streams.size() && s->streams[id].open) {
            const Lane* L = s->lanes[s->streams[id].lane].get();
            img = size_t(L->width) * L->height;
        }
    }
    if (img == 0) {
        delete r;
        return fail(PDFLOW_ERR_ARG, "no such stream");
    }
    // the frame is copied without the server's lock (the workers keep going)
    r->inten.assign(intensity, intensity + img);
    r->depth.assign(depth, depth + img);
    std::unique_lock<std::mutex> lk(s->mu);
    if (id >= s->streams.size() || !s->streams[id].open) {   // closed meanwhile
        delete r;
        return fail(PDFLOW_ERR_ARG, "no such stream");
    }
    Stream& st = s->streams[id];
    Lane* L = s->lanes[st.lane].get();
    r->id = s->next_id++;
    r->stream = id;
    r->slot = st.slot;
    r->frame = st.frames++;
    st.inflight++;
    s->requests[r->id] = r;
    L->pending.push_back(r);
    s->stats.submitted++;
    if (request_id) *request_id = r->id;
    lk.unlock();
    L->cv.notify_one();   // only this lane's worker has new work
    return PDFLOW_OK;
}

int pdflow_server_wait(pdflow_server* s, unsigned long long request_id, int timeout_ms, pdflow_request_info* info,
                       float* dx, float* dy, float* dz)
{
    if (!s) return fail(PDFLOW_ERR_ARG, "null argument");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(request_id);
    if (it == s->requests.end()) return fail(PDFLOW_ERR_ARG, "unknown request");
    Request* r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0)
        s->cv_done.wait(lk, ready);
    else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        return fail(PDFLOW_ERR_TIMEOUT, "request not done in time");
    if (info) {
        info->request_id = r->id;
        info->stream_id = r->stream;
        info->frame_index = r->frame;
        info->status = r->status;
        info->has_flow = r->has_flow ? 1 : 0;
        info->batch_pairs = r->batch_pairs;
        info->batch_fallbacks = r->batch_fallbacks;
        info->submit_ms = ms_since(s, r->t_submit);
        info->start_ms = ms_since(s, r->t_start);
        info->done_ms = ms_since(s, r->t_done);
    }
    s->requests.erase(it);
    lk.unlock();   // the request is ours now: its flow is copied without the lock
    if (r->has_flow) {
        const size_t N = r->dx.size();
        if (dx) std::memcpy(dx, r->dx.data(), N * 4);
        if (dy) std::memcpy(dy, r->dy.data(), N * 4);
        if (dz) std::memcpy(dz, r->dz.data(), N * 4);
    }
    delete r;
    return PDFLOW_OK;
}

int pdflow_server_replay(pdflow_server* s, const pdflow_replay_stream* streams, unsigned n_streams, double rate_hz,
                         unsigned long long seed, pdflow_request_info* info, double* late_ms, unsigned capacity,
                         unsigned* count)
{
    if (!s || !streams || !info || !late_ms || !count || !(rate_hz > 0.0)) return fail(PDFLOW_ERR_ARG, "bad argument");
    size_t total = 0;
    for (unsigned i = 0; i < n_streams; ++i) {
        if (streams[i].frames && (!streams[i].intensity || !streams[i].depth)) return fail(PDFLOW_ERR_ARG, "null frames");
        total += streams[i].frames;
    }
    if (total > capacity) return fail(PDFLOW_ERR_ARG, "more frames than result slots");
    struct Arrival {
        double t;   // seconds after the start
        unsigned stream, frame;
        bool operator>(const Arrival& o) const { return t > o.t; }
    };
    std::mt19937_64 rng(seed);
    std::exponential_distribution<double> gap(rate_hz);
    std::priority_queue<Arrival, std::vector<Arrival>, std::greater<Arrival>> due;
    for (unsigned i = 0; i < n_streams; ++i)
        if (streams[i].frames) due.push({gap(rng), i, 0});
    std::vector<unsigned long long> ids;
    ids.reserve(total);
    int rc = PDFLOW_OK;
    const auto t0 = Clock::now();
    while (!due.empty()) {
        const Arrival a = due.top();
        due.pop();
        std::this_thread::sleep_until(t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(a.t)));
        const pdflow_replay_stream& st = streams[a.stream];
        unsigned long long id = 0;
        late_ms[ids.size()] = std::chrono::duration<double, std::milli>(Clock::now() - t0).count() - a.t * 1e3;
        rc = pdflow_server_submit(s, st.stream_id, st.intensity[a.frame], st.depth[a.frame], &id);
        if (rc != PDFLOW_OK) break;
        ids.push_back(id);
        if (a.frame + 1 < st.frames) due.push({a.t + gap(rng), a.stream, a.frame + 1});
    }
    for (size_t m = 0; m < ids.size(); ++m) {
        const int w = pdflow_server_wait(s, ids[m], -1, &info[m], nullptr, nullptr, nullptr);
        if (w != PDFLOW_OK && rc == PDFLOW_OK) rc = w;
    }
    *count = unsigned(ids.size());
    return rc;
}

int pdflow_server_get_stats(pdflow_server* s, pdflow_server_stats* out)
{
    if (!s || !out) return fail(PDFLOW_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->lanes = unsigned(s->lanes.size());
    out->device_bytes = s->device_bytes;
    return PDFLOW_OK;
}

}  // extern "C"
