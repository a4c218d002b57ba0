// Batched rendering: job tables, the persistent launch, CUDA-graph replay and
// the launch-shape autotuner.  (No counterpart in the reference, which renders
// one frame per dispatch, src/render/Renderer.cpp:74-89.)
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/xenodon.h"
#include "xn_ctx.h"
#include "xn_internal.h"

namespace xn {

int make_launch(const Volume* v, int traversal, const xn_camera* cam, const xn_params* p, RenderLaunch& L);

namespace {

uint32_t traversal_mask(const xn_job* jobs, int n) {
    uint32_t m = 0;
    for (int i = 0; i < n; ++i) m |= 1u << (jobs[i].traversal & 7);
    return m;
}

int check_config(const xn_batch_config& c) {
    if (c.tile_width == XN_BATCH_PLAIN) return XN_OK;  // one single-frame launch per job
    if (c.tile_width != 4 && c.tile_width != 8 && c.tile_width != 16 && c.tile_width != 32)
        return fail(XN_ERR_ARG, "batch: tile_width must be 4, 8, 16 or 32 (or 0, one launch per frame)");
    if (c.block_threads == 0 || c.block_threads % 32 || c.block_threads > 1024)
        return fail(XN_ERR_ARG, "batch: block_threads must be a multiple of 32 up to 1024");

    return XN_OK;
}

// Builds header + jobs into `table`; returns the byte size.
int fill_table(Ctx* c, const xn_job* jobs, int n, uint32_t tile_w, void* table, uint64_t capacity_bytes,
               uint64_t* bytes_out, int* spec_out = nullptr) {
    const uint64_t need = sizeof(BatchHeader) + (uint64_t)n * sizeof(BatchJob);
    if (need > capacity_bytes) return fail(XN_ERR_ARG, "batch: %d jobs exceed the job table capacity", n);
    BatchHeader* h = static_cast<BatchHeader*>(table);
    BatchJob* out = reinterpret_cast<BatchJob*>(h + 1);
    const uint32_t tile_h = 32 / tile_w;
    unsigned long long tiles = 0;
    for (int i = 0; i < n; ++i) {
        const xn_job& j = jobs[i];
        if (!j.volume || !j.d_rgba) return fail(XN_ERR_ARG, "batch: job %d has no volume or output", i);
        const Volume* v = reinterpret_cast<const Volume*>(j.volume);
        if (v->ctx != c) return fail(XN_ERR_ARG, "batch: job %d uses a volume of another context", i);
        RenderLaunch L;
        int r = make_launch(v, j.traversal, &j.camera, &j.params, L);
        if (r) return r;
        L.d_rgba = j.d_rgba;
        out[i] = make_batch_job(L);
        out[i].tiles_x = (L.out_w + tile_w - 1) / tile_w;
        out[i].tiles_y = (L.out_h + tile_h - 1) / tile_h;
        out[i].tile_begin = tiles;
        tiles += (unsigned long long)out[i].tiles_x * out[i].tiles_y;
        const int sp = batch_spec(out[i]);
        out[i].form = sp;
        if (spec_out) *spec_out = i == 0 ? sp : (*spec_out == sp ? sp : XN_BATCH_ANY);
    }
    h->n_jobs = (uint32_t)n;
    h->pad = 0;
    h->total_tiles = tiles;
    *bytes_out = need;
    return XN_OK;
}

uint32_t resident_blocks(Ctx* c, const xn_batch_config& cfg) {
    int per_sm = batch_kernel_blocks_per_sm(cfg.tile_width, cfg.block_threads);
    if (per_sm < 1) per_sm = 1;
    if (cfg.blocks_per_sm && (int)cfg.blocks_per_sm < per_sm) per_sm = (int)cfg.blocks_per_sm;
    return (uint32_t)per_sm * (uint32_t)c->sm_count();
}

// 4x8 warp tiles, blocks of 256, no queue: the shape the autotuner picked most
// often (CT frames and the 1024^3 and 2048^3 gas fields, every traversal).
xn_batch_config default_config() { return xn_batch_config{4, 256, 0, 0}; }

// Pinned staging for the job tables of xn_render_batch (one per context; a
// new table is written only after the previous one was copied out).
int ensure_batch_staging(Ctx* c, uint64_t bytes) {
    if (!c->batch_copied && cudaEventCreateWithFlags(&c->batch_copied, cudaEventDisableTiming) != cudaSuccess)
        return fail(XN_ERR_CUDA, "batch: event");
    if (c->batch_host_bytes < bytes) {
        if (c->batch_host) {
            cudaEventSynchronize(c->batch_copied);
            cudaFreeHost(c->batch_host);
            c->batch_host = nullptr;
            c->batch_host_bytes = 0;
        }
        if (cudaHostAlloc(&c->batch_host, bytes, cudaHostAllocDefault) != cudaSuccess)
            return fail(XN_ERR_NOMEM, "batch: pinned job table");
        c->batch_host_bytes = bytes;
    }
    return XN_OK;
}

// Every launch gets a device job table and work counter of its own, allocated
// and freed in the order of its stream: launches on other streams (the render
// server runs several) never see them, and no launch waits for another.
// The kernel form (XN_BATCH_*) each job needs.
int forms_of(Ctx* c, const xn_job* jobs, int n, std::vector<int>& forms) {
    forms.resize(n);
    for (int i = 0; i < n; ++i) {
        if (!jobs[i].volume || !jobs[i].d_rgba) return fail(XN_ERR_ARG, "batch: job %d has no volume or output", i);
        const Volume* v = reinterpret_cast<const Volume*>(jobs[i].volume);
        if (v->ctx != c) return fail(XN_ERR_ARG, "batch: job %d uses a volume of another context", i);
        RenderLaunch L;
        int r = make_launch(v, jobs[i].traversal, &jobs[i].camera, &jobs[i].params, L);
        if (r) return r;
        forms[i] = batch_spec(make_batch_job(L));
    }
    return XN_OK;
}

bool generic_forced() {
    const char* generic = std::getenv("XN_BATCH_GENERIC");
    return generic && generic[0] == '1';
}

int render_batch_one(Ctx* c, const xn_job* jobs, int n, const xn_batch_config& cfg, cudaStream_t s);

// The plain form: every job through the single-frame kernels, one launch
// each, in order on the stream (the reference's one dispatch per frame,
// src/render/Renderer.cpp:74-89, with its launch shape and register budget).
int render_plain(Ctx* c, const xn_job* jobs, int n, cudaStream_t s) {
    for (int i = 0; i < n; ++i) {
        if (!jobs[i].volume || !jobs[i].d_rgba) return fail(XN_ERR_ARG, "batch: job %d has no volume or output", i);
        const Volume* v = reinterpret_cast<const Volume*>(jobs[i].volume);
        if (v->ctx != c) return fail(XN_ERR_ARG, "batch: job %d uses a volume of another context", i);
        RenderLaunch L;
        int r = make_launch(v, jobs[i].traversal, &jobs[i].camera, &jobs[i].params, L);
        if (r) return r;
        L.d_rgba = jobs[i].d_rgba;
        L.d_err_word = c->d_err;
        cudaError_t e = launch_render(L, s);
        if (e != cudaSuccess) return cuda_fail(e, "xn_render_batch: plain launch");
    }
    return XN_OK;
}

// A batch whose jobs need different kernel forms runs as one launch per form
// (each specialised, each over its own jobs, in the stream's order); with
// XN_BATCH_GENERIC=1 the generic form takes the whole batch in one launch.
int render_batch_locked(Ctx* c, const xn_job* jobs, int n, const xn_batch_config& cfg, cudaStream_t s) {
    if (cfg.tile_width == XN_BATCH_PLAIN) return render_plain(c, jobs, n, s);
    if (!generic_forced()) {
        std::vector<int> forms;
        int r = forms_of(c, jobs, n, forms);
        if (r) return r;
        bool mixed = false;
        for (int i = 1; i < n; ++i) mixed |= forms[i] != forms[0];
        if (mixed) {
            std::vector<xn_job> part;
            for (int f = 0; f < XN_BATCH_FORMS && !r; ++f) {
                part.clear();
                for (int i = 0; i < n; ++i)
                    if (forms[i] == f) part.push_back(jobs[i]);
                if (!part.empty()) r = render_batch_one(c, part.data(), (int)part.size(), cfg, s);
            }
            return r;
        }
    }
    return render_batch_one(c, jobs, n, cfg, s);
}

int render_batch_one(Ctx* c, const xn_job* jobs, int n, const xn_batch_config& cfg, cudaStream_t s) {
    const uint64_t cap = sizeof(BatchHeader) + (uint64_t)n * sizeof(BatchJob);
    int r = ensure_batch_staging(c, cap);
    if (r) return r;
    cudaError_t e = cudaEventSynchronize(c->batch_copied);  // the previous table left the staging buffer
    if (e != cudaSuccess) return cuda_fail(e, "xn_render_batch: staging");
    uint64_t bytes = 0;
    int spec = XN_BATCH_ANY;
    if ((r = fill_table(c, jobs, n, cfg.tile_width, c->batch_host, c->batch_host_bytes, &bytes, &spec))) return r;
    // XN_BATCH_GENERIC=1 keeps the generic form (same results)
    if (generic_forced()) spec = XN_BATCH_ANY;
    const uint64_t queue_off = (bytes + 255) & ~255ull;
    void* d = nullptr;
    e = cudaMallocAsync(&d, queue_off + 256, s);
    if (e != cudaSuccess) return cuda_fail(e, "xn_render_batch: job table");
    unsigned long long* queue = reinterpret_cast<unsigned long long*>(static_cast<char*>(d) + queue_off);
    e = cudaMemcpyAsync(d, c->batch_host, bytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(c->batch_copied, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(queue, 0, 8, s);
    const uint64_t total_tiles = static_cast<const BatchHeader*>(c->batch_host)->total_tiles;
    const uint32_t warps = cfg.block_threads / 32;
    const uint64_t grid = cfg.chunk ? resident_blocks(c, cfg) : (total_tiles + warps - 1) / warps;
    if (grid == 0) {
        cudaFreeAsync(d, s);
        return XN_OK;
    }
    if (grid > 0x7FFFFFFFull) {
        cudaFreeAsync(d, s);
        return fail(XN_ERR_ARG, "xn_render_batch: too many tiles for one grid; use a queue chunk >= 1");
    }
    if (e == cudaSuccess)
        e = launch_batch(d, queue, c->d_err, cfg.tile_width, cfg.block_threads, (uint32_t)grid, cfg.chunk, spec, s);
    const cudaError_t ef = cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = ef;
    return e == cudaSuccess ? XN_OK : cuda_fail(e, "xn_render_batch");
}

}  // namespace

int Ctx::sm_count() {
    if (sms <= 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || v <= 0) v = 1;
        sms = v;
    }
    return sms;
}

}  // namespace xn

using namespace xn;

XN_API int xn_render_batch(xn_ctx* h, const xn_job* jobs, int n, const xn_batch_config* cfg, void* stream) {
    if (!h || (!jobs && n)) return fail(XN_ERR_ARG, "xn_render_batch: NULL argument");
    if (n <= 0) return XN_OK;
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    xn_batch_config k = default_config();
    if (cfg) k = *cfg;
    else if (c->tuned_valid[traversal_mask(jobs, n)]) k = c->tuned[traversal_mask(jobs, n)];
    if ((r = check_config(k))) return r;
    return render_batch_locked(c, jobs, n, k, static_cast<cudaStream_t>(stream));
}

// Two rounds: every candidate launch shape -- the persistent kernel's tile /
// block / queue shapes and the plain form, one single-frame launch per job --
// is timed once on a sample of the jobs spread over the batch (at most 8), then
// the four fastest, the plain form always among them, are timed twice on the
// whole batch; the fastest of those wins.  The plain form being a finalist
// means the tuned batch does not lose to one launch per frame, up to timing
// noise.
XN_API int xn_autotune_batch(xn_ctx* h, const xn_job* jobs, int n, void* stream, xn_batch_config* best,
                             float* best_ms) {
    if (!h || !jobs || n <= 0) return fail(XN_ERR_ARG, "xn_autotune_batch: no jobs");
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return fail(XN_ERR_CUDA, "xn_autotune_batch: events");
    std::vector<xn_batch_config> cand;
    cand.push_back(xn_batch_config{XN_BATCH_PLAIN, 0, 0, 0});
    for (uint32_t tw : {4u, 8u, 16u, 32u})
        for (uint32_t bt : {64u, 128u, 256u})
            for (uint32_t ch : {0u, 1u, 2u, 4u})  // 0: one warp per tile over a full grid, no queue
                cand.push_back(xn_batch_config{tw, bt, 0, ch});
    std::vector<xn_job> sample;
    const int want = n < 8 ? n : 8;
    for (int i = 0; i < want; ++i) sample.push_back(jobs[(int)((int64_t)i * n / want)]);
    auto time_it = [&](const xn_batch_config& k, const xn_job* js, int m, int reps, float* ms_out) -> int {
        int rr = render_batch_locked(c, js, m, k, s);  // warm-up
        float best_t = 3.4e38f;
        for (int i = 0; i < reps && !rr; ++i) {
            cudaEventRecord(e0, s);
            rr = render_batch_locked(c, js, m, k, s);
            cudaEventRecord(e1, s);
            float ms = 0;
            if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
                rr = fail(XN_ERR_CUDA, "xn_autotune_batch: timing");
            best_t = std::min(best_t, ms);
        }
        *ms_out = best_t;
        return rr;
    };
    std::vector<std::pair<float, int>> score;
    for (size_t i = 0; i < cand.size() && !r; ++i) {
        float ms = 0;
        r = time_it(cand[i], sample.data(), (int)sample.size(), 1, &ms);
        score.emplace_back(ms, (int)i);
    }
    xn_batch_config winner = cand[0];
    float winner_ms = 3.4e38f;
    if (!r) {
        std::sort(score.begin(), score.end());
        std::vector<int> finalists;
        for (size_t i = 0; i < score.size() && finalists.size() < 3; ++i)
            if (score[i].second != 0) finalists.push_back(score[i].second);
        finalists.push_back(0);  // the plain form
        for (int idx : finalists) {
            float ms = 0;
            if ((r = time_it(cand[idx], jobs, n, 2, &ms))) break;
            if (ms < winner_ms) {
                winner_ms = ms;
                winner = cand[idx];
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r) return r;
    const uint32_t m = traversal_mask(jobs, n);
    c->tuned[m] = winner;
    c->tuned_valid[m] = 1;
    if (best) *best = winner;
    if (best_ms) *best_ms = winner_ms;
    return XN_OK;
}

// ------------------------------------------------------------------ graphs

// A batch graph captures one launch per kernel form, each over its own
// segment of the job table (a form without jobs exits at once), or with
// XN_BATCH_GENERIC=1 one generic launch over the whole table.
struct xn_batch_graph {
    Ctx* ctx;
    cudaStream_t stream;
    xn_batch_config cfg;
    bool split = true;
    int capacity;
    uint64_t seg_bytes;    // one form's segment: header + capacity jobs
    uint64_t table_bytes;  // all segments
    struct Slot {
        void* host = nullptr;
        void* dev = nullptr;
        unsigned long long* queue = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaEvent_t done = nullptr;
        bool pending = false;
    } slot[2];
    int next = 0;
};

namespace {

void destroy_graph(xn_batch_graph* g) {
    Ctx* c = g->ctx;
    for (auto& s : g->slot) {
        if (s.done) {
            cudaEventSynchronize(s.done);
            cudaEventDestroy(s.done);
        }
        if (s.exec) cudaGraphExecDestroy(s.exec);
        if (s.host) cudaFreeHost(s.host);
        c->device_free(s.dev, g->table_bytes);
        c->device_free(s.queue, 64 * XN_BATCH_FORMS);
    }
    delete g;
}

}  // namespace

XN_API int xn_batch_graph_create(xn_ctx* h, int capacity, const xn_batch_config* cfg, void* stream,
                                 xn_batch_graph** out) {
    if (!h || !out || capacity <= 0) return fail(XN_ERR_ARG, "xn_batch_graph_create: bad argument");
    *out = nullptr;
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    xn_batch_graph* g = new (std::nothrow) xn_batch_graph();
    if (!g) return fail(XN_ERR_NOMEM, "xn_batch_graph_create: out of host memory");
    g->ctx = c;
    g->stream = static_cast<cudaStream_t>(stream);
    g->cfg = cfg ? *cfg : default_config();
    if (g->cfg.tile_width == XN_BATCH_PLAIN) {
        delete g;
        return fail(XN_ERR_ARG, "xn_batch_graph_create: the plain form (one launch per frame) is not captured");
    }
    if (g->cfg.chunk == 0) g->cfg.chunk = 1;  // the tile count changes per replay: graphs use the queue form
    g->capacity = capacity;
    g->split = !generic_forced();
    g->seg_bytes = (sizeof(BatchHeader) + (uint64_t)capacity * sizeof(BatchJob) + 255) & ~255ull;
    g->table_bytes = g->seg_bytes * (g->split ? XN_BATCH_FORMS : 1);
    if ((r = check_config(g->cfg))) {
        delete g;
        return r;
    }
    const uint32_t blocks = resident_blocks(c, g->cfg);
    cudaStream_t cap = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    for (auto& sl : g->slot) {
        if (e != cudaSuccess || r) break;
        if ((e = cudaHostAlloc(&sl.host, g->table_bytes, cudaHostAllocDefault)) != cudaSuccess) break;
        std::memset(sl.host, 0, g->table_bytes);
        if ((r = c->device_alloc(&sl.dev, g->table_bytes, "xn_batch_graph_create: job table"))) break;
        if ((r = c->device_alloc(reinterpret_cast<void**>(&sl.queue), 64 * XN_BATCH_FORMS,
                                 "xn_batch_graph_create: queue")))
            break;
        if ((e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming)) != cudaSuccess) break;
        // capture: table upload, queue resets, one persistent launch per form
        if ((e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) break;
        cudaMemcpyAsync(sl.dev, sl.host, g->table_bytes, cudaMemcpyHostToDevice, cap);
        cudaMemsetAsync(sl.queue, 0, 64 * XN_BATCH_FORMS, cap);
        const int n_launch = g->split ? XN_BATCH_FORMS : 1;
        for (int f = 0; f < n_launch; ++f)
            launch_batch(static_cast<char*>(sl.dev) + f * g->seg_bytes, sl.queue + f * 8, c->d_err, g->cfg.tile_width,
                         g->cfg.block_threads, blocks, g->cfg.chunk, g->split ? f : XN_BATCH_ANY, cap);
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(cap, &graph);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&sl.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
    }
    if (cap) cudaStreamDestroy(cap);
    if (e != cudaSuccess || r) {
        destroy_graph(g);
        return r ? r : cuda_fail(e, "xn_batch_graph_create");
    }
    *out = g;
    return XN_OK;
}

XN_API int xn_batch_graph_launch(xn_batch_graph* g, const xn_job* jobs, int n) {
    if (!g || (!jobs && n)) return fail(XN_ERR_ARG, "xn_batch_graph_launch: NULL argument");
    if (n > g->capacity) return fail(XN_ERR_ARG, "xn_batch_graph_launch: %d jobs exceed the capacity %d", n, g->capacity);
    Ctx* c = g->ctx;
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    auto& sl = g->slot[g->next];
    if (sl.pending) cudaEventSynchronize(sl.done);  // this slot's previous batch has finished
    uint64_t bytes = 0;
    if (g->split) {
        std::vector<int> forms;
        if ((r = forms_of(c, jobs, n, forms))) return r;
        std::vector<xn_job> part;
        for (int f = 0; f < XN_BATCH_FORMS; ++f) {
            part.clear();
            for (int i = 0; i < n; ++i)
                if (forms[i] == f) part.push_back(jobs[i]);
            if ((r = fill_table(c, part.data(), (int)part.size(), g->cfg.tile_width,
                                static_cast<char*>(sl.host) + f * g->seg_bytes, g->seg_bytes, &bytes)))
                return r;
        }
    } else if ((r = fill_table(c, jobs, n, g->cfg.tile_width, sl.host, g->table_bytes, &bytes))) {
        return r;
    }
    cudaError_t e = cudaGraphLaunch(sl.exec, g->stream);
    if (e == cudaSuccess) e = cudaEventRecord(sl.done, g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "xn_batch_graph_launch");
    sl.pending = true;
    g->next ^= 1;
    return XN_OK;
}

XN_API int xn_batch_graph_destroy(xn_batch_graph* g) {
    if (!g) return XN_OK;
    std::lock_guard<std::mutex> lk(g->ctx->mu);
    g->ctx->activate();
    destroy_graph(g);
    return XN_OK;
}
