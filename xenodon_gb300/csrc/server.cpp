// Render server: continuous batching of render requests on one GPU.
//
// No counterpart in the reference (which renders one frame per dispatch from
// one camera script).  A worker thread keeps registered volumes resident in
// HBM with least-recently-used eviction, admits queued requests in arrival
// order while the HBM budget has room for their volume and output, renders
// each admitted set as one persistent batch (xn_render_batch) on one of
// several streams, and retires finished batches.  New requests are admitted as
// soon as a stream slot and memory are free, so their work overlaps on the
// device with the batches already running.  Latency is measured from submit to
// the result being in the caller's host buffer.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/xenodon.h"
#include "xn_ctx.h"

using xn::fail;

namespace {

using Clock = std::chrono::steady_clock;

// Frames of at least this many pixels fill the GPU in one launch (a GB300 holds
// 152 x 2048 resident threads).
constexpr uint64_t LARGE_FRAME = 1ull << 19;

struct ServerVolume {
    int kind = 0;
    std::vector<uint8_t> grid;
    uint32_t dim[3] = {0, 0, 0};
    std::vector<uint32_t> nodes;
    uint64_t side = 0;
    xn_volume* dev = nullptr;
    bool external = false;    // the caller's resident volume: never evicted or released here
    uint64_t dev_bytes = 0;   // measured once resident
    uint64_t estimate = 0;    // before the first upload
    uint64_t last_use = 0;
    int refs = 0;             // admitted requests using it
};

struct Request {
    uint64_t ticket = 0;
    uint32_t volume_id = 0;
    int traversal = 0;
    xn_camera cam{};
    xn_params params{};
    uint8_t* out = nullptr;
    uint64_t out_bytes = 0;
    void* d_out = nullptr;
    uint64_t staging_off = 0;
    Clock::time_point t_submit, t_done;
    int status = 1;  // 1 pending, 0 done, < 0 error
};

// A stream slot: FREE, RUNNING (its batch is on the GPU) or COPYING (the GPU
// is done; the copy thread moves the frames from the pinned staging buffer
// into the callers' buffers, then frees the slot).
enum class SlotState { FREE, RUNNING, COPYING };

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    void* staging = nullptr;
    uint64_t staging_bytes = 0;
    std::vector<Request*> reqs;
    SlotState state = SlotState::FREE;
};

}  // namespace

struct xn_server {
    xn_ctx* ctx = nullptr;
    xn_server_config cfg{};
    uint64_t budget = 0;
    uint64_t used = 0;  // resident volumes + outputs of admitted requests
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_copy;
    bool stop = false, stop_copier = false;
    std::thread worker, copier;
    std::deque<size_t> copy_queue;  // slots whose frames wait for the copy thread
    std::map<uint32_t, ServerVolume> volumes;
    std::deque<Request*> pending;
    std::unordered_map<uint64_t, Request*> requests;
    std::vector<Slot> slots;
    uint64_t next_ticket = 1, use_clock = 0;
    // statistics
    std::vector<double> latencies_ms;
    uint64_t rays = 0, batches = 0, batched_jobs = 0, uploads = 0, evictions = 0, failed = 0;
    Clock::time_point t_first{}, t_last{};
    bool any = false;

    void run();
    void copy_run();
    bool retire_finished();
    bool any_slot_in_use() const {
        for (const auto& sl : slots)
            if (sl.state != SlotState::FREE) return true;
        return false;
    }
    void launch_batch(Slot& slot);
    int make_resident(uint32_t id, ServerVolume& v, const std::vector<uint32_t>& protect);
};

namespace {

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

// Uploads a registered volume, evicting idle volumes (least recently used
// first) until it fits.  Called with the server mutex held.
int xn_server::make_resident(uint32_t id, ServerVolume& v, const std::vector<uint32_t>& protect) {
    if (v.dev) return XN_OK;
    const uint64_t need = v.dev_bytes ? v.dev_bytes : v.estimate;
    while (budget && used + need > budget) {
        uint32_t victim = 0;
        uint64_t oldest = ~0ull;
        bool found = false;
        for (auto& kv : volumes) {
            ServerVolume& o = kv.second;
            if (!o.dev || o.external || o.refs > 0 || kv.first == id) continue;
            if (std::find(protect.begin(), protect.end(), kv.first) != protect.end()) continue;
            if (o.last_use < oldest) {
                oldest = o.last_use;
                victim = kv.first;
                found = true;
            }
        }
        if (!found) return XN_ERR_BUDGET;
        ServerVolume& o = volumes[victim];
        xn_volume_release(o.dev);
        o.dev = nullptr;
        used -= o.dev_bytes;
        ++evictions;
    }
    int r = v.kind == XN_VOLUME_GRID
                ? xn_volume_upload_grid(ctx, v.grid.data(), v.dim[0], v.dim[1], v.dim[2], &v.dev)
                : xn_volume_upload_svo(ctx, v.nodes.data(), v.nodes.size() / 10, v.side, &v.dev);
    if (r) return r;
    xn_volume_info info;
    xn_volume_info_get(v.dev, &info);
    v.dev_bytes = info.device_bytes;
    used += v.dev_bytes;
    ++uploads;
    return XN_OK;
}

// Called with the server mutex held: slots whose batch finished on the GPU
// go to the copy thread (their device outputs are freed here, stream-ordered);
// a batch that failed on the device fails its requests.
bool xn_server::retire_finished() {
    bool any_retired = false;
    for (size_t k = 0; k < slots.size(); ++k) {
        Slot& slot = slots[k];
        if (slot.state != SlotState::RUNNING) continue;
        const cudaError_t q_state = cudaEventQuery(slot.done);
        if (q_state == cudaErrorNotReady) continue;
        for (Request* q : slot.reqs) {
            cudaFreeAsync(q->d_out, slot.stream);
            q->d_out = nullptr;
            used -= q->out_bytes;
            volumes[q->volume_id].refs--;
        }
        if (q_state != cudaSuccess) {
            for (Request* q : slot.reqs) {
                q->status = XN_ERR_CUDA;
                ++failed;
            }
            slot.reqs.clear();
            slot.state = SlotState::FREE;
            cv_done.notify_all();
        } else {
            slot.state = SlotState::COPYING;
            copy_queue.push_back(k);
            cv_copy.notify_one();
        }
        any_retired = true;
    }
    return any_retired;
}

// The copy thread: pinned staging -> callers' buffers, outside the mutex, so
// the worker keeps launching while frames are copied out.
void xn_server::copy_run() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv_copy.wait(lk, [&] { return stop_copier || !copy_queue.empty(); });
        if (copy_queue.empty()) break;  // stopping and nothing left
        const size_t k = copy_queue.front();
        copy_queue.pop_front();
        Slot& slot = slots[k];
        std::vector<Request*> reqs = slot.reqs;
        lk.unlock();
        for (Request* q : reqs)
            std::memcpy(q->out, static_cast<uint8_t*>(slot.staging) + q->staging_off, q->out_bytes);
        const auto now = Clock::now();
        lk.lock();
        for (Request* q : reqs) {
            q->t_done = now;
            q->status = 0;
            latencies_ms.push_back(ms_between(q->t_submit, now));
            rays += (uint64_t)q->params.output_region.width * q->params.output_region.height;
            t_last = now;
        }
        slot.reqs.clear();
        slot.state = SlotState::FREE;
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

void xn_server::launch_batch(Slot& slot) {
    std::vector<Request*> batch;
    std::vector<uint32_t> protect;
    while (!pending.empty() && (int)batch.size() < cfg.max_batch_jobs) {
        Request* q = pending.front();
        auto it = volumes.find(q->volume_id);
        if (it == volumes.end()) {  // the volume was removed after submit
            pending.pop_front();
            q->status = XN_ERR_STATE;
            ++failed;
            cv_done.notify_all();
            continue;
        }
        ServerVolume& v = it->second;
        const uint64_t vol_need = v.dev ? 0 : (v.dev_bytes ? v.dev_bytes : v.estimate);
        if (budget && (v.dev ? v.dev_bytes : vol_need) + q->out_bytes > budget) {
            // this volume and frame can never fit, whatever is evicted
            pending.pop_front();
            q->status = XN_ERR_BUDGET;
            ++failed;
            cv_done.notify_all();
            continue;
        }
        if (budget && used + q->out_bytes > budget) break;
        int r = make_resident(q->volume_id, v, protect);
        if (r == XN_ERR_BUDGET) break;  // wait for memory: later requests stay behind (arrival order)
        if (!r && budget && used + q->out_bytes > budget) break;
        void* d = nullptr;
        if (!r && cudaMallocAsync(&d, q->out_bytes, slot.stream) != cudaSuccess) r = XN_ERR_NOMEM;
        pending.pop_front();
        if (r) {
            q->status = r;
            ++failed;
            cv_done.notify_all();
            continue;
        }
        q->d_out = d;
        used += q->out_bytes;
        v.refs++;
        v.last_use = ++use_clock;
        protect.push_back(q->volume_id);
        batch.push_back(q);
    }
    if (batch.empty()) return;
    std::vector<xn_job> jobs(batch.size());
    uint64_t staging = 0;
    for (size_t i = 0; i < batch.size(); ++i) {
        Request* q = batch[i];
        jobs[i] = xn_job{volumes[q->volume_id].dev, q->traversal, q->cam, q->params, q->d_out};
        q->staging_off = staging;
        staging += (q->out_bytes + 255) & ~255ull;
    }
    if (slot.staging_bytes < staging) {
        if (slot.staging) cudaFreeHost(slot.staging);
        slot.staging = nullptr;
        slot.staging_bytes = 0;
        if (cudaHostAlloc(&slot.staging, staging, cudaHostAllocDefault) == cudaSuccess) slot.staging_bytes = staging;
    }
    // frames big enough to fill the GPU alone go to the single-frame kernels
    // (they gain nothing from the batch kernel); the rest share one batch
    std::vector<xn_job> small;
    int r = slot.staging ? XN_OK : XN_ERR_NOMEM;
    for (size_t i = 0; !r && i < jobs.size(); ++i) {
        const xn_rect& o = jobs[i].params.output_region;
        if ((uint64_t)o.width * o.height >= LARGE_FRAME)
            r = xn_render_device(ctx, jobs[i].volume, jobs[i].traversal, &jobs[i].camera, &jobs[i].params,
                                 jobs[i].d_rgba, nullptr, nullptr, slot.stream);
        else
            small.push_back(jobs[i]);
    }
    if (!r && !small.empty()) r = xn_render_batch(ctx, small.data(), (int)small.size(), nullptr, slot.stream);
    for (size_t i = 0; !r && i < batch.size(); ++i)
        if (cudaMemcpyAsync(static_cast<uint8_t*>(slot.staging) + batch[i]->staging_off, batch[i]->d_out,
                            batch[i]->out_bytes, cudaMemcpyDeviceToHost, slot.stream) != cudaSuccess)
            r = XN_ERR_CUDA;
    if (!r && cudaEventRecord(slot.done, slot.stream) != cudaSuccess) r = XN_ERR_CUDA;
    if (r) {  // fail the whole batch
        cudaStreamSynchronize(slot.stream);
        for (Request* q : batch) {
            cudaFreeAsync(q->d_out, slot.stream);
            q->d_out = nullptr;
            used -= q->out_bytes;
            volumes[q->volume_id].refs--;
            q->status = r;
            ++failed;
        }
        cv_done.notify_all();
        return;
    }
    slot.reqs = std::move(batch);
    slot.state = SlotState::RUNNING;
    ++batches;
    batched_jobs += slot.reqs.size();
}

void xn_server::run() {
    cudaSetDevice(reinterpret_cast<xn::Ctx*>(ctx)->device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        retire_finished();
        if (stop && !any_slot_in_use()) break;
        if (!stop && !pending.empty()) {
            for (auto& slot : slots) {
                if (pending.empty()) break;
                if (slot.state == SlotState::FREE) launch_batch(slot);
            }
        }
        bool running = false;
        for (auto& sl : slots) running |= sl.state == SlotState::RUNNING;
        if (running || any_slot_in_use()) {
            // poll the batches on the GPU; wake early for new requests or a freed slot
            cv_work.wait_for(lk, std::chrono::microseconds(100));
        } else if (pending.empty() && !stop) {
            cv_work.wait(lk, [&] { return stop || !pending.empty(); });
        }
    }
}

XN_API int xn_server_create(xn_ctx* ctx, const xn_server_config* cfg, xn_server** out) {
    if (!ctx || !out) return fail(XN_ERR_ARG, "xn_server_create: NULL argument");
    *out = nullptr;
    xn_server* s = new (std::nothrow) xn_server();
    if (!s) return fail(XN_ERR_NOMEM, "xn_server_create: out of host memory");
    s->ctx = ctx;
    s->cfg = cfg ? *cfg : xn_server_config{0, 256, 3};
    if (s->cfg.max_batch_jobs <= 0) s->cfg.max_batch_jobs = 256;
    if (s->cfg.streams <= 0) s->cfg.streams = 3;
    uint64_t used = 0, budget = 0;
    xn_ctx_memory(ctx, &used, &budget);
    s->budget = s->cfg.hbm_budget ? s->cfg.hbm_budget : budget;
    xn::Ctx* c = reinterpret_cast<xn::Ctx*>(ctx);
    if (cudaSetDevice(c->device) != cudaSuccess) {
        delete s;
        return fail(XN_ERR_CUDA, "xn_server_create: cudaSetDevice");
    }
    s->slots.resize(s->cfg.streams);
    for (auto& sl : s->slots) {
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            xn_server_destroy(s);
            return fail(XN_ERR_CUDA, "xn_server_create: streams");
        }
    }
    s->worker = std::thread([s] { s->run(); });
    s->copier = std::thread([s] { s->copy_run(); });
    *out = s;
    return XN_OK;
}

XN_API int xn_server_destroy(xn_server* s) {
    if (!s) return XN_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (Request* q : s->pending) q->status = XN_ERR_STATE;
        s->pending.clear();
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();  // returns once every slot is free again
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop_copier = true;
    }
    s->cv_copy.notify_all();
    if (s->copier.joinable()) s->copier.join();
    for (auto& kv : s->volumes)
        if (kv.second.dev && !kv.second.external) xn_volume_release(kv.second.dev);
    for (auto& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.staging) cudaFreeHost(sl.staging);
    }
    for (auto& kv : s->requests) delete kv.second;
    delete s;
    return XN_OK;
}

XN_API int xn_server_add_grid(xn_server* s, uint32_t id, const uint8_t* rgba, uint32_t dx, uint32_t dy, uint32_t dz) {
    if (!s || !rgba || !dx || !dy || !dz) return fail(XN_ERR_ARG, "xn_server_add_grid: bad argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->volumes.count(id)) return fail(XN_ERR_ARG, "xn_server_add_grid: volume %u exists", id);
    ServerVolume& v = s->volumes[id];
    v.kind = XN_VOLUME_GRID;
    v.grid.assign(rgba, rgba + (uint64_t)dx * dy * dz * 4);
    v.dim[0] = dx;
    v.dim[1] = dy;
    v.dim[2] = dz;
    v.estimate = (uint64_t)dx * dy * dz * 4;
    return XN_OK;
}

XN_API int xn_server_add_svo(xn_server* s, uint32_t id, const uint32_t* nodes, uint64_t n, uint64_t side) {
    if (!s || !nodes || !n) return fail(XN_ERR_ARG, "xn_server_add_svo: bad argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->volumes.count(id)) return fail(XN_ERR_ARG, "xn_server_add_svo: volume %u exists", id);
    ServerVolume& v = s->volumes[id];
    v.kind = XN_VOLUME_SVO;
    v.nodes.assign(nodes, nodes + n * 10);
    v.side = side;
    // the resident size of the device layout (svo_layout.cu): 68 bytes per
    // internal node and 32 per leaf; a leaf root keeps the 40-byte node
    uint64_t n_inner = 0;
    for (uint64_t i = 0; i < n; ++i) n_inner += nodes[i * 10 + 9] < 0x80000000u ? 1 : 0;
    v.estimate = n_inner ? n_inner * 68 + (n - n_inner) * 32 : n * 40;
    return XN_OK;
}

XN_API int xn_server_add_volume(xn_server* s, uint32_t id, xn_volume* volume) {
    if (!s || !volume) return fail(XN_ERR_ARG, "xn_server_add_volume: NULL argument");
    xn_volume_info info;
    int r = xn_volume_info_get(volume, &info);
    if (r) return r;
    if (reinterpret_cast<xn::Volume*>(volume)->ctx != reinterpret_cast<xn::Ctx*>(s->ctx))
        return fail(XN_ERR_ARG, "xn_server_add_volume: volume belongs to another context");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->volumes.count(id)) return fail(XN_ERR_ARG, "xn_server_add_volume: volume %u exists", id);
    if (s->budget && s->used + info.device_bytes > s->budget)
        return fail(XN_ERR_BUDGET, "xn_server_add_volume: %llu bytes exceed the HBM budget",
                    (unsigned long long)info.device_bytes);
    ServerVolume& v = s->volumes[id];
    v.kind = info.kind;
    v.dev = volume;
    v.external = true;
    v.dev_bytes = info.device_bytes;
    v.estimate = info.device_bytes;
    s->used += info.device_bytes;
    return XN_OK;
}

XN_API int xn_server_submit(xn_server* s, uint32_t volume_id, int traversal, const xn_camera* cam,
                            const xn_params* params, uint8_t* out_rgba, uint64_t* ticket) {
    if (!s || !cam || !params || !out_rgba || !ticket) return fail(XN_ERR_ARG, "xn_server_submit: NULL argument");
    if (params->output_region.width == 0 || params->output_region.height == 0)
        return fail(XN_ERR_ARG, "xn_server_submit: empty output region");
    Request* q = new (std::nothrow) Request();
    if (!q) return fail(XN_ERR_NOMEM, "xn_server_submit: out of host memory");
    q->volume_id = volume_id;
    q->traversal = traversal;
    q->cam = *cam;
    q->params = *params;
    q->out = out_rgba;
    q->out_bytes = (uint64_t)params->output_region.width * params->output_region.height * 4;
    q->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            delete q;
            return fail(XN_ERR_STATE, "xn_server_submit: the server is stopping");
        }
        auto it = s->volumes.find(volume_id);
        if (it == s->volumes.end()) {
            delete q;
            return fail(XN_ERR_ARG, "xn_server_submit: no volume %u", volume_id);
        }
        const bool grid = it->second.kind == XN_VOLUME_GRID;
        if (traversal < XN_DDA || traversal > XN_SVO_ROPE || (traversal == XN_DDA) != grid) {
            delete q;
            return fail(XN_ERR_ARG, "xn_server_submit: traversal %d does not fit volume %u", traversal, volume_id);
        }
        if (s->budget && q->out_bytes > s->budget) {
            delete q;
            return fail(XN_ERR_BUDGET, "xn_server_submit: the frame alone exceeds the HBM budget");
        }
        q->ticket = s->next_ticket++;
        if (!s->any) {
            s->t_first = q->t_submit;
            s->any = true;
        }
        s->requests[q->ticket] = q;
        s->pending.push_back(q);
        *ticket = q->ticket;
    }
    s->cv_work.notify_one();
    return XN_OK;
}

XN_API int xn_server_wait(xn_server* s, uint64_t ticket, double timeout_s, double* latency_ms) {
    if (!s) return fail(XN_ERR_ARG, "xn_server_wait: NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) return fail(XN_ERR_ARG, "xn_server_wait: unknown ticket %llu", (unsigned long long)ticket);
    Request* q = it->second;
    auto pred = [&] { return q->status != 1; };
    if (timeout_s < 0) s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
        return fail(XN_ERR_STATE, "xn_server_wait: ticket %llu not done yet", (unsigned long long)ticket);
    const int st = q->status;
    if (latency_ms) *latency_ms = st == 0 ? ms_between(q->t_submit, q->t_done) : 0.0;
    s->requests.erase(it);
    delete q;
    return st == 0 ? XN_OK : fail(st, "xn_server_wait: request %llu failed (%d)", (unsigned long long)ticket, st);
}

XN_API int xn_server_stats(xn_server* s, xn_server_metrics* out) {
    if (!s || !out) return fail(XN_ERR_ARG, "xn_server_stats: NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof *out);
    out->completed = s->latencies_ms.size();
    out->failed = s->failed;
    out->batches = s->batches;
    out->mean_batch = s->batches ? (double)s->batched_jobs / s->batches : 0.0;
    out->uploads = s->uploads;
    out->evictions = s->evictions;
    out->rays = s->rays;
    out->hbm_used = s->used;
    if (!s->latencies_ms.empty()) {
        std::vector<double> l = s->latencies_ms;
        std::sort(l.begin(), l.end());
        auto pct = [&](double p) {
            size_t k = (size_t)(p * (l.size() - 1) + 0.5);
            return l[std::min(k, l.size() - 1)];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = l.back();
        const double span = ms_between(s->t_first, s->t_last);
        out->mrays_per_s = span > 0 ? (double)s->rays / (span * 1000.0) : 0.0;
    }
    return XN_OK;
}
