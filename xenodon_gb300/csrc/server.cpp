// Render server: continuous batching of render requests on one GPU.
//
// No counterpart in the reference (which renders one frame per dispatch from
// one camera script, src/main_loop.cpp:230-258).  A worker thread keeps
// registered volumes resident in HBM with least-recently-used eviction and
// admits requests as the HBM budget allows, by size:
//
//  - small frames (below fold_max_pixels) are folded into a persistent kernel
//    while it runs: the worker appends each one to a job ring in device memory
//    and raises the ring's published tile count (render.cu fold_kernel), on a
//    high-priority stream of that ring.  The kernel claims tiles as they are
//    published and flags each finished job in mapped host memory; the worker
//    then copies that frame out at once, without waiting for the rest.  The
//    kernel leaves after a short idle time (every device-side wait is
//    bounded) and says so in the same mapped memory; that ring, like one
//    whose slots are used up, is closed and the other ring takes new jobs
//    (on its own stream, so its kernel does not queue behind the leaving
//    one); jobs a ring held when its kernel left are published again;
//  - large frames (each fills the GPU alone) run through the single-frame
//    kernels, each on one of `streams` low-priority streams (a few frames in
//    flight, so one frame's last blocks overlap the next frame's first), and
//    are copied out on that stream as soon as they are done.
//
// The persistent kernel runs on a high-priority stream: the block scheduler
// places its blocks ahead of the pending blocks of the large frames' grids
// as those retire, so a small frame does not wait for a large frame to end.
// A large frame can also be launched in bands of rows (band_pixels), which
// bounds how long a newly launched persistent kernel waits to be placed.
// Output buffers come from a pool, so admission does not allocate; a copy
// thread moves finished frames from pinned staging into the callers'
// buffers.  Latency is measured from submit to the frame in the caller's
// buffer.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/xenodon.h"
#include "xn_ctx.h"
#include "xn_internal.h"

namespace xn {
int make_launch(const Volume* v, int traversal, const xn_camera* cam, const xn_params* p, RenderLaunch& L);
}  // namespace xn

using xn::fail;

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint32_t FOLD_TILE_W = 8;  // warp tiles of 8 x 4 pixels
constexpr int FOLD_RINGS = 2;

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
    void* d_out = nullptr;       // from the device pool once admitted
    uint64_t d_bytes = 0;
    void* staging = nullptr;     // pinned, while being copied out
    uint64_t staging_bytes = 0;
    cudaEvent_t copied = nullptr;
    bool large = false;
    Clock::time_point t_submit, t_launch, t_flagged, t_copied, t_done;
    int status = 1;  // 1 pending, 0 done, < 0 error
};

// Buffers of power-of-two sizes, kept for reuse (device or pinned host).
struct Pool {
    bool device = true;
    std::multimap<uint64_t, void*> free;
    std::vector<std::pair<void*, uint64_t>> all;
    static uint64_t round(uint64_t b) {
        uint64_t r = 64 << 10;
        while (r < b) r <<= 1;
        return r;
    }
    void* get(uint64_t bytes, uint64_t* got) {
        const uint64_t r = round(bytes);
        auto it = free.find(r);
        if (it != free.end()) {
            void* p = it->second;
            free.erase(it);
            *got = r;
            return p;
        }
        void* p = nullptr;
        const cudaError_t e = device ? cudaMalloc(&p, r) : cudaHostAlloc(&p, r, cudaHostAllocDefault);
        if (e != cudaSuccess) return nullptr;
        all.emplace_back(p, r);
        *got = r;
        return p;
    }
    void put(void* p, uint64_t r) {
        if (p) free.emplace(r, p);
    }
    void release() {
        for (auto& a : all) device ? (void)cudaFree(a.first) : (void)cudaFreeHost(a.first);
        all.clear();
        free.clear();
    }
};

// One folding ring: device control words, job slots and per-slot tile
// counts; mapped host done flags; pinned mirrors of what is copied up.
struct FoldRing {
    xn::FoldCtl* d_ctl = nullptr;
    xn::BatchJob* d_ring = nullptr;
    uint32_t* d_done_tiles = nullptr;
    uint32_t* h_done = nullptr;           // mapped pinned host memory: one flag per slot, then the leaving flag
    uint32_t* d_done_alias = nullptr;     // its device address
    xn::BatchJob* h_ring = nullptr;       // pinned
    unsigned long long* h_pub = nullptr;  // pinned: the published count after each slot
    uint32_t* h_one = nullptr;            // pinned constant 1 (the closed flag)
    cudaEvent_t ready = nullptr, ended = nullptr;
    cudaStream_t stream = nullptr;        // high priority; one per ring, so a new kernel never queues behind a leaving one
    uint32_t n = 0;
    unsigned long long tiles = 0;
    bool launched = false, closed = false;
    std::vector<Request*> req;
    std::vector<char> collected;
};

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

}  // namespace

struct xn_server {
    xn_ctx* ctx = nullptr;
    xn::Ctx* c = nullptr;
    xn_server_config cfg{};
    uint64_t budget = 0;
    uint64_t used = 0;  // resident volumes + outputs of admitted requests
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_copy;
    bool stop = false, stop_copier = false;
    std::thread worker, copier;
    std::map<uint32_t, ServerVolume> volumes;
    std::deque<Request*> pending_small, pending_large;
    std::unordered_map<uint64_t, Request*> requests;
    std::vector<Request*> copying;    // D2H copies in flight (an event each)
    std::deque<Request*> copy_queue;  // copied to staging; the copy thread finishes them
    std::vector<Request*> large_inflight;
    cudaStream_t ctl_stream = nullptr, copy_stream = nullptr;
    std::vector<cudaStream_t> large_streams;  // low priority, one per large frame in flight
    size_t next_large = 0;
    FoldRing rings[FOLD_RINGS];
    int cur_ring = 0;
    Pool dev_pool, host_pool;
    std::vector<cudaEvent_t> event_pool;
    uint64_t next_ticket = 1, use_clock = 0;
    // statistics
    std::vector<double> latencies_ms;
    uint64_t rays = 0, launches = 0, launched_jobs = 0, folded = 0, fold_launches = 0, republished = 0;
    uint64_t uploads = 0, evictions = 0, failed = 0;
    Clock::time_point t_first{}, t_last{};
    bool any = false;
    // XN_SERVER_TRACE=<path>: one line per completed request, written when
    // the server is destroyed (ticket, large, pixels, traversal, then the ms
    // from submit to launch, launch to done on the GPU, to copied, to done)
    std::string trace_path;
    std::vector<std::string> trace;
    // XN_FOLD_THREADS=32|128: threads per block of the persistent kernel
    uint32_t fold_threads = 128;

    void run();
    void copy_run();
    int make_resident(uint32_t id, ServerVolume& v);
    bool admit(Request* q);
    void unadmit(Request* q);
    void fail_request(Request* q, int code);
    void start_copy(Request* q, cudaStream_t s);
    bool poll_rings();
    bool poll_copies();
    void publish_small();
    void launch_large();
    int reset_ring(FoldRing& r);
    bool busy() const;
    cudaEvent_t take_event() {
        if (!event_pool.empty()) {
            cudaEvent_t e = event_pool.back();
            event_pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        return e;
    }
};

// Uploads a registered volume, evicting idle volumes (least recently used
// first) until it fits.  Called with the server mutex held.
int xn_server::make_resident(uint32_t id, ServerVolume& v) {
    if (v.dev) return XN_OK;
    const uint64_t need = v.dev_bytes ? v.dev_bytes : v.estimate;
    while (budget && used + need > budget) {
        uint32_t victim = 0;
        uint64_t oldest = ~0ull;
        bool found = false;
        for (auto& kv : volumes) {
            ServerVolume& o = kv.second;
            if (!o.dev || o.external || o.refs > 0 || kv.first == id) continue;
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

void xn_server::fail_request(Request* q, int code) {
    q->status = code;
    ++failed;
    cv_done.notify_all();
}

// Volume resident, output buffer taken from the pool, memory counted.  False
// when the request must wait for memory (it stays queued); a request that can
// never run fails.
bool xn_server::admit(Request* q) {
    auto it = volumes.find(q->volume_id);
    if (it == volumes.end()) {  // the volume was removed after submit
        fail_request(q, XN_ERR_STATE);
        return true;
    }
    ServerVolume& v = it->second;
    const uint64_t vol_need = v.dev_bytes ? v.dev_bytes : v.estimate;
    if (budget && (v.dev ? v.dev_bytes : vol_need) + q->out_bytes > budget) {
        fail_request(q, XN_ERR_BUDGET);  // this volume and frame never fit, whatever is evicted
        return true;
    }
    if (budget && used + q->out_bytes > budget) return false;
    int r = make_resident(q->volume_id, v);
    if (r == XN_ERR_BUDGET) return false;  // wait for memory
    if (!r && budget && used + q->out_bytes > budget) return false;
    if (!r) {
        q->d_out = dev_pool.get(q->out_bytes, &q->d_bytes);
        if (!q->d_out) r = XN_ERR_NOMEM;
    }
    if (r) {
        fail_request(q, r);
        return true;
    }
    used += q->out_bytes;
    v.refs++;
    v.last_use = ++use_clock;
    return true;
}

void xn_server::unadmit(Request* q) {
    if (!q->d_out) return;
    dev_pool.put(q->d_out, q->d_bytes);
    q->d_out = nullptr;
    used -= q->out_bytes;
    volumes[q->volume_id].refs--;
}

// Frame -> pinned staging on stream s (after the work queued there); the
// output buffer goes back to the pool once the copy has been seen done.
void xn_server::start_copy(Request* q, cudaStream_t s) {
    q->staging = host_pool.get(q->out_bytes, &q->staging_bytes);
    q->copied = take_event();
    cudaError_t e = q->staging && q->copied ? cudaSuccess : cudaErrorMemoryAllocation;
    if (e == cudaSuccess) e = cudaMemcpyAsync(q->staging, q->d_out, q->out_bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaEventRecord(q->copied, s);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(s);
        host_pool.put(q->staging, q->staging_bytes);
        q->staging = nullptr;
        if (q->copied) event_pool.push_back(q->copied);
        q->copied = nullptr;
        unadmit(q);
        fail_request(q, XN_ERR_CUDA);
        return;
    }
    copying.push_back(q);
}

int xn_server::reset_ring(FoldRing& r) {
    cudaError_t e = cudaMemsetAsync(r.d_ring, 0xFF, (size_t)cfg.max_batch_jobs * sizeof(xn::BatchJob), ctl_stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(r.d_ctl, 0, sizeof(xn::FoldCtl), ctl_stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(r.d_done_tiles, 0, (size_t)cfg.max_batch_jobs * 4, ctl_stream);
    std::memset(r.h_done, 0, ((size_t)cfg.max_batch_jobs + 1) * 4);
    r.n = 0;
    r.tiles = 0;
    r.launched = r.closed = false;
    std::fill(r.req.begin(), r.req.end(), nullptr);
    std::fill(r.collected.begin(), r.collected.end(), 0);
    return e == cudaSuccess ? XN_OK : XN_ERR_CUDA;
}

// Finished jobs go to their copies; a ring whose kernel has left has its
// unfinished jobs queued again (in their order, ahead of newer ones) and is
// made ready for reuse.
bool xn_server::poll_rings() {
    bool progress = false;
    for (int ri = 0; ri < FOLD_RINGS; ++ri) {
        FoldRing& r = rings[ri];
        if (!r.launched) continue;
        for (uint32_t k = 0; k < r.n; ++k) {
            if (r.collected[k]) continue;
            if (reinterpret_cast<volatile uint32_t*>(r.h_done)[k]) {
                r.collected[k] = 1;
                r.req[k]->t_flagged = Clock::now();
                start_copy(r.req[k], copy_stream);
                progress = true;
            }
        }
        const cudaError_t q = cudaEventQuery(r.ended);
        if (q == cudaErrorNotReady) continue;
        // the kernel has left: anything not flagged done by now never will be
        std::vector<Request*> again;
        for (uint32_t k = 0; k < r.n; ++k) {
            if (r.collected[k]) continue;
            if (reinterpret_cast<volatile uint32_t*>(r.h_done)[k] && q == cudaSuccess) {
                r.collected[k] = 1;
                r.req[k]->t_flagged = Clock::now();
                start_copy(r.req[k], copy_stream);
            } else if (q == cudaSuccess) {
                again.push_back(r.req[k]);
            } else {
                unadmit(r.req[k]);
                fail_request(r.req[k], XN_ERR_CUDA);
            }
        }
        republished += again.size();
        for (auto it = again.rbegin(); it != again.rend(); ++it) pending_small.push_front(*it);
        if (reset_ring(r) != XN_OK) {
            for (Request* x : again) {
                pending_small.erase(std::find(pending_small.begin(), pending_small.end(), x));
                unadmit(x);
                fail_request(x, XN_ERR_CUDA);
            }
        }
        if (cur_ring != ri && rings[cur_ring].closed) cur_ring = ri;
        progress = true;
    }
    return progress;
}

// Copies that reached pinned memory go to the copy thread.
bool xn_server::poll_copies() {
    bool progress = false;
    for (size_t i = 0; i < copying.size();) {
        Request* q = copying[i];
        const cudaError_t e = cudaEventQuery(q->copied);
        if (e == cudaErrorNotReady) {
            ++i;
            continue;
        }
        copying[i] = copying.back();
        copying.pop_back();
        q->t_copied = Clock::now();
        if (q->large) q->t_flagged = q->t_copied;  // kernel and copy share the frame's stream
        event_pool.push_back(q->copied);
        q->copied = nullptr;
        unadmit(q);
        if (e != cudaSuccess) {
            host_pool.put(q->staging, q->staging_bytes);
            q->staging = nullptr;
            fail_request(q, XN_ERR_CUDA);
        } else {
            copy_queue.push_back(q);
            cv_copy.notify_one();
        }
        progress = true;
    }
    // a large frame stops being in flight once its copy was seen done
    for (size_t i = 0; i < large_inflight.size();) {
        if (std::find(copying.begin(), copying.end(), large_inflight[i]) == copying.end()) {
            large_inflight[i] = large_inflight.back();
            large_inflight.pop_back();
            progress = true;
        } else {
            ++i;
        }
    }
    return progress;
}

// Small frames into the current ring, while it has slots and memory allows.
void xn_server::publish_small() {
    while (!pending_small.empty()) {
        FoldRing& r = rings[cur_ring];
        if (r.launched && !r.closed && reinterpret_cast<volatile uint32_t*>(r.h_done)[cfg.max_batch_jobs]) {
            // its kernel has decided to leave and takes no new tiles: what it
            // still holds is published again once it has ended
            r.closed = true;
        }
        if (r.closed) {
            // the other ring takes over once its kernel has left and it was reset
            const int other = (cur_ring + 1) % FOLD_RINGS;
            if (rings[other].launched || rings[other].closed) return;
            cur_ring = other;
            continue;
        }
        Request* q = pending_small.front();
        if (!q->d_out) {
            if (!admit(q)) return;
            if (q->status != 1) {
                pending_small.pop_front();
                continue;
            }
        }
        pending_small.pop_front();
        xn::RenderLaunch L;
        const xn::Volume* v = reinterpret_cast<const xn::Volume*>(volumes[q->volume_id].dev);
        int rc = xn::make_launch(v, q->traversal, &q->cam, &q->params, L);
        if (rc) {
            unadmit(q);
            fail_request(q, rc);
            continue;
        }
        L.d_rgba = q->d_out;
        const uint32_t k = r.n;
        xn::BatchJob j = xn::make_batch_job(L);
        j.tiles_x = (L.out_w + FOLD_TILE_W - 1) / FOLD_TILE_W;
        j.tiles_y = (L.out_h + 32 / FOLD_TILE_W - 1) / (32 / FOLD_TILE_W);
        j.tile_begin = r.tiles;
        j.form = xn::batch_spec(j);
        r.h_ring[k] = j;
        r.tiles += (unsigned long long)j.tiles_x * j.tiles_y;
        r.h_pub[k] = r.tiles;
        r.req[k] = q;
        // the job, then the count that covers it: one stream, in that order
        cudaError_t e = cudaMemcpyAsync(r.d_ring + k, r.h_ring + k, sizeof(xn::BatchJob), cudaMemcpyHostToDevice,
                                        ctl_stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&r.d_ctl->published, r.h_pub + k, 8, cudaMemcpyHostToDevice, ctl_stream);
        if (e == cudaSuccess && !r.launched) {
            e = cudaEventRecord(r.ready, ctl_stream);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(r.stream, r.ready, 0);
            // fold_blocks_per_sm x 4 warps per SM, in blocks of fold_threads
            const uint32_t blocks =
                (uint32_t)c->sm_count() * std::max(1u, cfg.fold_blocks_per_sm) * (128u / fold_threads);
            if (e == cudaSuccess)
                e = xn::launch_fold(r.d_ctl, r.d_ring, (uint32_t)cfg.max_batch_jobs, r.d_done_tiles, r.d_done_alias,
                                    c->d_err, FOLD_TILE_W, fold_threads, blocks,
                                    (unsigned long long)cfg.fold_idle_us * 1000ull,
                                    r.stream);
            if (e == cudaSuccess) e = cudaEventRecord(r.ended, r.stream);
            if (e == cudaSuccess) {
                r.launched = true;
                ++fold_launches;
                ++launches;
            }
        }
        if (e != cudaSuccess) {  // the ring is unusable: fail what it holds
            cudaStreamSynchronize(ctl_stream);
            cudaStreamSynchronize(r.stream);
            for (uint32_t i = 0; i <= k; ++i)
                if (r.req[i] && !r.collected[i]) {
                    unadmit(r.req[i]);
                    fail_request(r.req[i], XN_ERR_CUDA);
                }
            reset_ring(r);
            return;
        }
        r.n = k + 1;
        q->t_launch = Clock::now();
        ++folded;
        ++launched_jobs;
        if (r.n == (uint32_t)cfg.max_batch_jobs) {  // full: close it; the other ring continues
            cudaMemcpyAsync(&r.d_ctl->closed, r.h_one, 4, cudaMemcpyHostToDevice, ctl_stream);
            r.closed = true;
        }
    }
}

// Large frames through the single-frame kernels, a few in flight.
void xn_server::launch_large() {
    while (!pending_large.empty() && (int)large_inflight.size() < cfg.streams) {
        Request* q = pending_large.front();
        if (!q->d_out) {
            if (!admit(q)) return;
            if (q->status != 1) {
                pending_large.pop_front();
                continue;
            }
        }
        pending_large.pop_front();
        // in bands of rows of about fold_max_pixels each: between two bands
        // the GPU drains, and the persistent kernel's waiting blocks (higher
        // priority) are placed before the next band's, so a small frame waits
        // at most one band, not a whole large frame (the pixels are the same:
        // every band keeps the frame's display region)
        const xn_rect o = q->params.output_region;
        const uint32_t band =
            cfg.band_pixels ? (uint32_t)std::max<uint64_t>(1, cfg.band_pixels / o.width) : o.height;
        cudaStream_t st = large_streams[next_large];
        next_large = (next_large + 1) % large_streams.size();
        int r = XN_OK;
        for (uint32_t y0 = 0; y0 < o.height && !r; y0 += band) {
            xn_params p = q->params;
            p.output_region.y = o.y + (int32_t)y0;
            p.output_region.height = std::min(band, o.height - y0);
            r = xn_render_device(ctx, volumes[q->volume_id].dev, q->traversal, &q->cam, &p,
                                 static_cast<uint8_t*>(q->d_out) + (uint64_t)y0 * o.width * 4, nullptr, nullptr, st);
        }
        if (r) {
            unadmit(q);
            fail_request(q, r);
            continue;
        }
        ++launches;
        ++launched_jobs;
        q->t_launch = Clock::now();
        start_copy(q, st);
        if (q->status == 1) large_inflight.push_back(q);
    }
}

bool xn_server::busy() const {
    if (!copying.empty() || !copy_queue.empty() || !large_inflight.empty()) return true;
    for (const auto& r : rings)
        if (r.launched) return true;
    return false;
}

// The copy thread: pinned staging -> callers' buffers, outside the mutex.
void xn_server::copy_run() {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv_copy.wait(lk, [&] { return stop_copier || !copy_queue.empty(); });
        if (copy_queue.empty()) break;  // stopping and nothing left
        Request* q = copy_queue.front();
        copy_queue.pop_front();
        lk.unlock();
        std::memcpy(q->out, q->staging, q->out_bytes);
        const auto now = Clock::now();
        lk.lock();
        host_pool.put(q->staging, q->staging_bytes);
        q->staging = nullptr;
        q->t_done = now;
        q->status = 0;
        latencies_ms.push_back(ms_between(q->t_submit, now));
        if (!trace_path.empty()) {
            char line[256];
            std::snprintf(line, sizeof line, "%llu %d %llu %d %.3f %.3f %.3f %.3f", (unsigned long long)q->ticket,
                          q->large ? 1 : 0,
                          (unsigned long long)q->params.output_region.width * q->params.output_region.height,
                          q->traversal, ms_between(q->t_submit, q->t_launch), ms_between(q->t_launch, q->t_flagged),
                          ms_between(q->t_flagged, q->t_copied), ms_between(q->t_copied, now));
            trace.emplace_back(line);
        }
        rays += (uint64_t)q->params.output_region.width * q->params.output_region.height;
        t_last = now;
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

void xn_server::run() {
    cudaSetDevice(c->device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        poll_rings();
        poll_copies();
        if (stop) {
            // close the open rings so their kernels leave once drained
            for (auto& r : rings)
                if (r.launched && !r.closed) {
                    cudaMemcpyAsync(&r.d_ctl->closed, r.h_one, 4, cudaMemcpyHostToDevice, ctl_stream);
                    r.closed = true;
                }
            if (!busy()) break;
        } else {
            publish_small();
            launch_large();
        }
        if (busy()) {
            // poll the work on the GPU; wake early for new requests
            cv_work.wait_for(lk, std::chrono::microseconds(20));
        } else if (!stop && pending_small.empty() && pending_large.empty()) {
            cv_work.wait(lk, [&] { return stop || !pending_small.empty() || !pending_large.empty(); });
        } else if (!stop) {
            cv_work.wait_for(lk, std::chrono::microseconds(200));  // waiting for memory
        }
    }
    // requests a ring handed back after the stop are not rendered
    for (auto* dq : {&pending_small, &pending_large}) {
        for (Request* q : *dq) {
            unadmit(q);
            q->status = XN_ERR_STATE;
        }
        dq->clear();
    }
    cv_done.notify_all();
}

XN_API int xn_server_create(xn_ctx* ctx, const xn_server_config* cfg, xn_server** out) {
    if (!ctx || !out) return fail(XN_ERR_ARG, "xn_server_create: NULL argument");
    *out = nullptr;
    xn_server* s = new (std::nothrow) xn_server();
    if (!s) return fail(XN_ERR_NOMEM, "xn_server_create: out of host memory");
    s->ctx = ctx;
    s->c = reinterpret_cast<xn::Ctx*>(ctx);
    s->cfg = cfg ? *cfg : xn_server_config{};
    if (s->cfg.max_batch_jobs <= 0) s->cfg.max_batch_jobs = 1024;
    if (s->cfg.max_batch_jobs > (1 << 16)) s->cfg.max_batch_jobs = 1 << 16;
    if (s->cfg.streams <= 0) s->cfg.streams = 2;
    if (s->cfg.streams > 16) s->cfg.streams = 16;
    if (s->cfg.fold_max_pixels == 0) s->cfg.fold_max_pixels = 1ull << 19;
    if (s->cfg.fold_idle_us == 0) s->cfg.fold_idle_us = 300;
    if (s->cfg.fold_blocks_per_sm == 0) s->cfg.fold_blocks_per_sm = 2;
    if (s->cfg.fold_blocks_per_sm > 4) s->cfg.fold_blocks_per_sm = 4;
    s->host_pool.device = false;
    if (const char* tp = std::getenv("XN_SERVER_TRACE")) s->trace_path = tp;
    if (const char* ft = std::getenv("XN_FOLD_THREADS")) s->fold_threads = std::atoi(ft) == 32 ? 32u : 128u;
    uint64_t used = 0, budget = 0;
    xn_ctx_memory(ctx, &used, &budget);
    s->budget = s->cfg.hbm_budget ? s->cfg.hbm_budget : budget;
    if (cudaSetDevice(s->c->device) != cudaSuccess) {
        delete s;
        return fail(XN_ERR_CUDA, "xn_server_create: cudaSetDevice");
    }
    int lo = 0, hi = 0;  // numerically lower is more urgent
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    bool ok = cudaStreamCreateWithFlags(&s->ctl_stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithPriority(&s->copy_stream, cudaStreamNonBlocking, hi) == cudaSuccess;
    for (int i = 0; ok && i < s->cfg.streams; ++i) {
        cudaStream_t st = nullptr;
        ok = cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, lo) == cudaSuccess;
        if (ok) s->large_streams.push_back(st);
    }
    const uint64_t cap = (uint64_t)s->cfg.max_batch_jobs;
    for (auto& r : s->rings) {
        if (!ok) break;
        ok = cudaMalloc(reinterpret_cast<void**>(&r.d_ctl), sizeof(xn::FoldCtl)) == cudaSuccess &&
             cudaMalloc(reinterpret_cast<void**>(&r.d_ring), cap * sizeof(xn::BatchJob)) == cudaSuccess &&
             cudaMalloc(reinterpret_cast<void**>(&r.d_done_tiles), cap * 4) == cudaSuccess &&
             cudaStreamCreateWithPriority(&r.stream, cudaStreamNonBlocking, hi) == cudaSuccess &&
             cudaHostAlloc(reinterpret_cast<void**>(&r.h_done), (cap + 1) * 4, cudaHostAllocMapped) == cudaSuccess &&
             cudaHostGetDevicePointer(reinterpret_cast<void**>(&r.d_done_alias), r.h_done, 0) == cudaSuccess &&
             cudaHostAlloc(reinterpret_cast<void**>(&r.h_ring), cap * sizeof(xn::BatchJob), cudaHostAllocDefault) ==
                 cudaSuccess &&
             cudaHostAlloc(reinterpret_cast<void**>(&r.h_pub), cap * 8, cudaHostAllocDefault) == cudaSuccess &&
             cudaHostAlloc(reinterpret_cast<void**>(&r.h_one), 4, cudaHostAllocDefault) == cudaSuccess &&
             cudaEventCreateWithFlags(&r.ready, cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&r.ended, cudaEventDisableTiming) == cudaSuccess;
        if (!ok) break;
        *r.h_one = 1;
        r.req.assign(cap, nullptr);
        r.collected.assign(cap, 0);
        ok = s->reset_ring(r) == XN_OK;
    }
    if (ok) ok = cudaStreamSynchronize(s->ctl_stream) == cudaSuccess;
    if (!ok) {
        xn_server_destroy(s);
        return fail(XN_ERR_CUDA, "xn_server_create: streams and rings");
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
        for (auto* dq : {&s->pending_small, &s->pending_large})
            for (Request* q : *dq) {
                s->unadmit(q);
                q->status = XN_ERR_STATE;
            }
        s->pending_small.clear();
        s->pending_large.clear();
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();  // returns once nothing is in flight
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop_copier = true;
    }
    s->cv_copy.notify_all();
    if (s->copier.joinable()) s->copier.join();
    s->cv_done.notify_all();
    cudaSetDevice(s->c->device);
    for (cudaStream_t st : {s->ctl_stream, s->copy_stream})
        if (st) cudaStreamSynchronize(st);
    for (auto& r : s->rings)
        if (r.stream) cudaStreamSynchronize(r.stream);
    for (cudaStream_t st : s->large_streams) cudaStreamSynchronize(st);
    for (auto& kv : s->volumes)
        if (kv.second.dev && !kv.second.external) xn_volume_release(kv.second.dev);
    for (auto& r : s->rings) {
        cudaFree(r.d_ctl);
        cudaFree(r.d_ring);
        cudaFree(r.d_done_tiles);
        if (r.h_done) cudaFreeHost(r.h_done);
        if (r.h_ring) cudaFreeHost(r.h_ring);
        if (r.h_pub) cudaFreeHost(r.h_pub);
        if (r.h_one) cudaFreeHost(r.h_one);
        if (r.ready) cudaEventDestroy(r.ready);
        if (r.ended) cudaEventDestroy(r.ended);
        if (r.stream) cudaStreamDestroy(r.stream);
    }
    s->dev_pool.release();
    s->host_pool.release();
    for (cudaEvent_t e : s->event_pool) cudaEventDestroy(e);
    for (cudaStream_t st : {s->ctl_stream, s->copy_stream})
        if (st) cudaStreamDestroy(st);
    for (cudaStream_t st : s->large_streams) cudaStreamDestroy(st);
    for (auto& kv : s->requests) delete kv.second;
    if (!s->trace_path.empty()) {
        if (std::FILE* f = std::fopen(s->trace_path.c_str(), "a")) {
            std::fprintf(f, "# ticket large pixels traversal submit->launch launch->gpu_done gpu_done->copied "
                            "copied->done (ms)\n");
            for (const auto& l : s->trace) std::fprintf(f, "%s\n", l.c_str());
            std::fclose(f);
        }
    }
    delete s;
    return XN_OK;
}

namespace {

// A newly registered volume is uploaded at once when the budget has room, so
// requests do not wait for it; otherwise on first use.
void upload_if_room(xn_server* s, uint32_t id) {
    ServerVolume& v = s->volumes[id];
    if (!s->budget || s->used + v.estimate <= s->budget) s->make_resident(id, v);
}

}  // namespace

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
    upload_if_room(s, id);
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
    upload_if_room(s, id);
    return XN_OK;
}

XN_API int xn_server_add_volume(xn_server* s, uint32_t id, xn_volume* volume) {
    if (!s || !volume) return fail(XN_ERR_ARG, "xn_server_add_volume: NULL argument");
    xn_volume_info info;
    int r = xn_volume_info_get(volume, &info);
    if (r) return r;
    if (reinterpret_cast<xn::Volume*>(volume)->ctx != s->c)
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
    q->large = (uint64_t)params->output_region.width * params->output_region.height >= s->cfg.fold_max_pixels;
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
        (q->large ? s->pending_large : s->pending_small).push_back(q);
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
    out->batches = s->launches;
    out->mean_batch = s->launches ? (double)s->launched_jobs / s->launches : 0.0;
    out->uploads = s->uploads;
    out->evictions = s->evictions;
    out->rays = s->rays;
    out->hbm_used = s->used;
    out->folded = s->folded;
    out->fold_launches = s->fold_launches;
    out->republished = s->republished;
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
