// Job engine behind vvpt_submit / vvpt_poll / vvpt_wait / vvpt_render_batch.
//
// One worker thread per context owns a fixed pool of path slots and runs the
// wavefront kernels as CUDA graphs over every admitted job at once: the work
// items of all jobs form one global hand-out sequence (hand-out ranges in the
// job table), so the regeneration kernel refills a finished slot with the
// next item of whichever job owns it, and each stage's queue holds paths of
// every live job. Between graph replays the worker admits queued jobs (FIFO,
// within the device budget), and finishes jobs whose work items are all done
// (per-job reduce into the caller's outputs). A completion thread waits for
// each finished job's reduce, copies host outputs and wakes waiters, so the
// worker never blocks on a copy.
//
// A job's result equals vvpt_render of the same request bit for bit: its
// per-(pixel, batch) RNG streams and sums do not depend on which slot or
// iteration runs them, and the final reduce sums batches in order.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.h"

namespace vvpt {

namespace {

constexpr uint32_t kMaxJobSlots = 1024;
constexpr uint32_t kMaxRanges = 4096;

// Device-side counters of the engine's job table.
struct TableCounters {
    unsigned long long next_item;
    unsigned long long total_items;
    uint32_t num_ranges;
    uint32_t idle_count;
    uint32_t pad[2];
};

// What the worker reads back after each graph replay.
struct Readback {
    uint32_t counters[C_COUNT];
    uint32_t done[kMaxJobSlots];
    unsigned long long next_item;
};

struct EJob {
    vvpt_job id = 0;
    vvpt_scene *scene = nullptr;
    RenderParams hp{};
    vvpt_outputs out{};
    uint32_t state = VVPT_JOB_QUEUED;
    vvpt_status status = VVPT_OK;
    std::string error;
    double submit_ms = 0, start_ms = 0, end_ms = 0;
    uint64_t paths = 0;
    uint64_t bytes_results = 0, bytes_staging = 0;
    int slot = -1;
    uint64_t admit_seq = 0;    // graph launches before admission
    float4 *results = nullptr; // 3 arrays of total_items
    float4 *staging = nullptr; // device images for host outputs
    cudaEvent_t done_ev = nullptr;
};

size_t job_result_bytes(const RenderParams &hp) { return 3 * aligned256((size_t)hp.total_items * sizeof(float4)); }

size_t job_staging_bytes(const RenderParams &hp, const vvpt_outputs &o)
{
    if (o.on_device)
        return 0;
    const size_t img = aligned256((size_t)hp.width * hp.height * sizeof(float4));
    size_t n = 0;
    for (const float *p : {o.radiance, o.albedo, o.normal, o.radiance_m2})
        n += p ? img : 0;
    return n;
}

}  // namespace

struct Engine {
    vvpt_ctx *ctx = nullptr;
    int device = 0;
    std::thread worker, completer;
    std::mutex m;
    std::condition_variable cv_work, cv_done, cv_complete;
    bool stop = false;
    bool completer_stop = false;
    bool broken = false;
    std::string broken_msg;
    std::deque<std::shared_ptr<EJob>> pending;
    std::deque<std::shared_ptr<EJob>> completing;
    std::unordered_map<vvpt_job, std::shared_ptr<EJob>> jobs;
    uint64_t next_id = 1;
    uint64_t fixed_bytes = 0, used_bytes = 0;
    bool ready = false; // device state built (or failed: broken)

    // device state (worker thread only)
    cudaStream_t stream = nullptr, copy_stream = nullptr;
    cudaMemPool_t pool = nullptr;
    DevBuf state_buf, queue_buf, table_buf;
    PathState ps{};
    Queues q{};
    JobTable jt{};
    JobView *d_jobs = nullptr;
    unsigned long long *d_range_begin = nullptr;
    uint32_t *d_range_job = nullptr;
    uint32_t *d_done = nullptr;
    TableCounters *d_tc = nullptr;
    Readback *rb_host = nullptr; // pinned, 2 entries
    cudaEvent_t rb_ev[2] = {nullptr, nullptr};
    cudaGraphExec_t exec = nullptr;
    uint32_t slots = 0;
    int graph_iters = 8;

    double now_ms() const;
    void fail_job_locked(const std::shared_ptr<EJob> &j, vvpt_status st, const std::string &msg);
    bool init_device(std::string &err);
    void release_device();
    void run();
    void complete_loop();
};

double Engine::now_ms() const
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - ctx->created).count();
}

void Engine::fail_job_locked(const std::shared_ptr<EJob> &j, vvpt_status st, const std::string &msg)
{
    j->state = VVPT_JOB_FAILED;
    j->status = st;
    j->error = msg;
    j->end_ms = now_ms();
    j->scene->jobs_in_flight.fetch_sub(1);
    cv_done.notify_all();
}

bool Engine::init_device(std::string &err)
{
    auto ck = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess) {
            cudaGetLastError();
            err = std::string(what) + ": " + cudaGetErrorString(e);
            return false;
        }
        return true;
    };
    if (!ck(cudaSetDevice(device), "cudaSetDevice"))
        return false;
    if (!ck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream") ||
        !ck(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking), "stream"))
        return false;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (!ck(cudaMemPoolCreate(&pool, &props), "cudaMemPoolCreate"))
        return false;
    uint64_t keep = ~0ull; // keep freed blocks for the next jobs
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);

    const vvpt_tuning &t = ctx->tuning;
    slots = t.slots ? t.slots : (1u << 20);
    slots = std::max<uint32_t>(slots, 32u);
    graph_iters = t.iterations_per_graph ? (int)t.iterations_per_graph : 8;
    graph_iters = (graph_iters + 1) & ~1;
    if (!ck(state_buf.alloc(path_state_bytes(slots)), "cudaMalloc path state") ||
        !ck(queue_buf.alloc(queue_bytes(slots)), "cudaMalloc queues"))
        return false;
    ps = carve_path_state(state_buf.as<char>(), slots);
    q = carve_queues(queue_buf.as<char>(), slots);
    const size_t tb = aligned256(kMaxJobSlots * sizeof(JobView)) + aligned256(kMaxRanges * 8) +
                      aligned256(kMaxRanges * 4) + aligned256(kMaxJobSlots * 4) + aligned256(sizeof(TableCounters)) +
                      aligned256((size_t)slots * 4);
    if (!ck(table_buf.alloc(tb), "cudaMalloc job table"))
        return false;
    char *base = table_buf.as<char>();
    auto take = [&](size_t b) {
        char *p = base;
        base += aligned256(b);
        return p;
    };
    d_jobs = (JobView *)take(kMaxJobSlots * sizeof(JobView));
    d_range_begin = (unsigned long long *)take(kMaxRanges * 8);
    d_range_job = (uint32_t *)take(kMaxRanges * 4);
    d_done = (uint32_t *)take(kMaxJobSlots * 4);
    d_tc = (TableCounters *)take(sizeof(TableCounters));
    uint32_t *d_idle = (uint32_t *)take((size_t)slots * 4);
    fixed_bytes = path_state_bytes(slots) + queue_bytes(slots) + tb;
    jt.jobs = d_jobs;
    jt.range_begin = d_range_begin;
    jt.range_job = d_range_job;
    jt.item_done = d_done;
    jt.next_item = &d_tc->next_item;
    jt.total_items = &d_tc->total_items;
    jt.num_ranges = &d_tc->num_ranges;
    jt.idle = d_idle;
    jt.idle_count = &d_tc->idle_count;
    if (!ck(cudaMemsetAsync(table_buf.ptr, 0, tb, stream), "clear job table"))
        return false;
    launch_init_slots(q, ps, jt, slots, stream);
    if (!ck(cudaGetLastError(), "launch init"))
        return false;
    if (!ck(cudaMallocHost(&rb_host, 2 * sizeof(Readback)), "cudaMallocHost readback"))
        return false;
    for (int k = 0; k < 2; k++)
        if (!ck(cudaEventCreateWithFlags(&rb_ev[k], cudaEventDisableTiming), "event"))
            return false;

    LaunchShape shape;
    shape.block = t.threads_per_block ? (int)t.threads_per_block : 256;
    shape.grid = std::max(1, ctx->num_sms * (t.blocks_per_sm ? (int)t.blocks_per_sm : 4));
    cudaGraph_t graph;
    if (!ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture"))
        return false;
    for (int it = 0; it < graph_iters; it++)
        launch_iteration(jt, ps, q, it & 1, shape, stream);
    if (!ck(cudaStreamEndCapture(stream, &graph), "end capture"))
        return false;
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (!ck(e, "graph instantiate"))
        return false;
    return ck(cudaStreamSynchronize(stream), "engine init");
}

void Engine::release_device()
{
    cudaSetDevice(device);
    if (stream)
        cudaStreamSynchronize(stream);
    if (copy_stream)
        cudaStreamSynchronize(copy_stream);
    if (exec)
        cudaGraphExecDestroy(exec);
    for (auto &e : rb_ev)
        if (e)
            cudaEventDestroy(e);
    if (rb_host)
        cudaFreeHost(rb_host);
    state_buf.release();
    queue_buf.release();
    table_buf.release();
    if (pool)
        cudaMemPoolDestroy(pool);
    if (stream)
        cudaStreamDestroy(stream);
    if (copy_stream)
        cudaStreamDestroy(copy_stream);
}

void Engine::run()
{
    std::string err;
    const bool ok = init_device(err);
    {
        std::lock_guard<std::mutex> lk(m);
        ready = true;
        if (!ok) {
            broken = true;
            broken_msg = "engine start: " + err;
        }
        cv_done.notify_all();
    }
    std::vector<std::shared_ptr<EJob>> running;
    std::vector<int> free_slots;
    for (int s = (int)kMaxJobSlots - 1; s >= 0; s--)
        free_slots.push_back(s);
    std::vector<unsigned long long> rbeg;
    std::vector<uint32_t> rjob;
    unsigned long long total = 0;   // end of the last hand-out range
    unsigned long long floor_ = 0;  // every item below was handed out
    unsigned long long rb_total[2] = {0, 0};
    uint64_t rb_seq[2] = {0, 0};
    uint64_t launch_seq = 0;
    int cur = 0;
    bool have_prev = false;

    for (;;) {
        bool admitted = false;
        {
            std::unique_lock<std::mutex> lk(m);
            if (broken) {
                for (auto &j : pending)
                    fail_job_locked(j, VVPT_ERR_DEVICE, broken_msg);
                pending.clear();
            }
            while (!stop && pending.empty() && running.empty())
                cv_work.wait(lk);
            if (stop)
                break;
            // admission, first come first served
            while (!pending.empty() && !broken) {
                std::shared_ptr<EJob> j = pending.front();
                const RenderParams &hp = j->hp;
                const size_t img = (size_t)hp.width * hp.height * sizeof(float4);
                if (hp.batches == 0 || hp.depth == 0 || hp.total_items == 0) {
                    // nothing traced: outputs cleared, as vvpt_render
                    pending.pop_front();
                    j->state = VVPT_JOB_RUNNING;
                    j->start_ms = now_ms();
                    bool okc = true;
                    for (float *p : {j->out.radiance, j->out.albedo, j->out.normal, j->out.radiance_m2}) {
                        if (!p)
                            continue;
                        if (j->out.on_device)
                            okc &= cudaMemsetAsync(p, 0, img, stream) == cudaSuccess;
                        else
                            std::memset(p, 0, img);
                    }
                    cudaEventCreateWithFlags(&j->done_ev, cudaEventDisableTiming);
                    cudaEventRecord(j->done_ev, stream);
                    if (!okc)
                        fail_job_locked(j, VVPT_ERR_DEVICE, "clear outputs failed");
                    else {
                        completing.push_back(j);
                        cv_complete.notify_one();
                    }
                    continue;
                }
                if (free_slots.empty() || rbeg.size() >= kMaxRanges)
                    break;
                const uint64_t need = j->bytes_results + j->bytes_staging;
                if (ctx->budget_bytes && fixed_bytes + used_bytes + need > ctx->budget_bytes)
                    break;
                void *res = nullptr, *stg = nullptr;
                cudaError_t e1 = cudaMallocFromPoolAsync(&res, j->bytes_results, pool, stream);
                cudaError_t e2 = e1 == cudaSuccess && j->bytes_staging
                                     ? cudaMallocFromPoolAsync(&stg, j->bytes_staging, pool, stream)
                                     : cudaSuccess;
                if (e1 != cudaSuccess || e2 != cudaSuccess) {
                    cudaGetLastError();
                    if (res)
                        cudaFreeAsync(res, stream);
                    if (!running.empty())
                        break; // retry once running jobs free memory
                    pending.pop_front();
                    fail_job_locked(j, VVPT_ERR_OOM, "device memory exhausted for the job's batch sums");
                    continue;
                }
                pending.pop_front();
                j->results = (float4 *)res;
                j->staging = (float4 *)stg;
                j->slot = free_slots.back();
                free_slots.pop_back();
                j->state = VVPT_JOB_RUNNING;
                j->start_ms = now_ms();
                j->admit_seq = launch_seq;
                used_bytes += need;
                JobView jv;
                jv.scene = j->scene->view;
                jv.params = hp;
                const size_t rbytes = aligned256((size_t)hp.total_items * sizeof(float4));
                jv.results.rad = j->results;
                jv.results.alb = (float4 *)((char *)j->results + rbytes);
                jv.results.nrm = (float4 *)((char *)j->results + 2 * rbytes);
                // pageable source: copied out before the call returns
                cudaMemcpyAsync(d_jobs + j->slot, &jv, sizeof(jv), cudaMemcpyHostToDevice, stream);
                cudaMemsetAsync(d_done + j->slot, 0, sizeof(uint32_t), stream);
                rbeg.push_back(total);
                rjob.push_back((uint32_t)j->slot);
                total += hp.total_items;
                running.push_back(j);
                admitted = true;
            }
        }
        if (broken) {
            std::lock_guard<std::mutex> lk(m);
            for (auto &j : running)
                fail_job_locked(j, VVPT_ERR_DEVICE, broken_msg);
            running.clear();
            continue;
        }
        if (admitted) {
            // drop ranges that were handed out completely
            size_t drop = 0;
            while (drop + 1 < rbeg.size() && rbeg[drop + 1] <= floor_)
                drop++;
            if (drop) {
                rbeg.erase(rbeg.begin(), rbeg.begin() + drop);
                rjob.erase(rjob.begin(), rjob.begin() + drop);
            }
            cudaMemcpyAsync(d_range_begin, rbeg.data(), rbeg.size() * 8, cudaMemcpyHostToDevice, stream);
            cudaMemcpyAsync(d_range_job, rjob.data(), rjob.size() * 4, cudaMemcpyHostToDevice, stream);
            launch_admit(q, jt, total, (uint32_t)rbeg.size(), stream);
        }
        if (running.empty()) {
            have_prev = false;
            continue;
        }
        cudaError_t e = cudaGraphLaunch(exec, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(rb_host[cur].counters, q.counters, C_COUNT * 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(rb_host[cur].done, d_done, kMaxJobSlots * 4, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&rb_host[cur].next_item, &d_tc->next_item, 8, cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess)
            e = cudaEventRecord(rb_ev[cur], stream);
        rb_total[cur] = total;
        rb_seq[cur] = ++launch_seq;
        const int prev = cur ^ 1;
        cur ^= 1;
        if (e != cudaSuccess) {
            std::lock_guard<std::mutex> lk(m);
            broken = true;
            broken_msg = std::string("graph launch: ") + cudaGetErrorString(e);
            continue;
        }
        if (!have_prev) {
            have_prev = true;
            continue;
        }
        e = cudaEventSynchronize(rb_ev[prev]);
        const Readback &r = rb_host[prev];
        if (e != cudaSuccess || r.counters[C_ERR]) {
            std::lock_guard<std::mutex> lk(m);
            broken = true;
            broken_msg = e != cudaSuccess ? std::string("engine: ") + cudaGetErrorString(e)
                                          : "device status word set: " + std::to_string(r.counters[C_ERR]);
            continue;
        }
        floor_ = std::max(floor_, std::min(r.next_item, rb_total[prev]));
        // finish jobs whose work items are all done
        for (size_t i = 0; i < running.size();) {
            std::shared_ptr<EJob> j = running[i];
            // a readback queued before the job's admission holds the slot's
            // previous count
            if (rb_seq[prev] <= j->admit_seq || r.done[j->slot] < j->hp.total_items) {
                i++;
                continue;
            }
            const RenderParams &hp = j->hp;
            const size_t npix = (size_t)hp.width * hp.height;
            const size_t rbytes = aligned256((size_t)hp.total_items * sizeof(float4));
            BatchResults br;
            br.rad = j->results;
            br.alb = (float4 *)((char *)j->results + rbytes);
            br.nrm = (float4 *)((char *)j->results + 2 * rbytes);
            float4 *dst[4];
            float *src[4] = {j->out.radiance, j->out.albedo, j->out.normal, j->out.radiance_m2};
            size_t off = 0;
            for (int k = 0; k < 4; k++) {
                if (!src[k])
                    dst[k] = nullptr;
                else if (j->out.on_device)
                    dst[k] = reinterpret_cast<float4 *>(src[k]);
                else {
                    dst[k] = (float4 *)((char *)j->staging + off);
                    off += aligned256(npix * sizeof(float4));
                }
            }
            launch_reduce(hp, br, dst[0], dst[1], dst[2], dst[3], stream);
            cudaFreeAsync(j->results, stream);
            j->results = nullptr;
            cudaEventCreateWithFlags(&j->done_ev, cudaEventDisableTiming);
            cudaEventRecord(j->done_ev, stream);
            free_slots.push_back(j->slot);
            running.erase(running.begin() + i);
            std::lock_guard<std::mutex> lk(m);
            used_bytes -= j->bytes_results;
            completing.push_back(j);
            cv_complete.notify_one();
        }
    }
    // shutdown: fail what did not finish
    {
        std::lock_guard<std::mutex> lk(m);
        for (auto &j : running)
            fail_job_locked(j, VVPT_ERR_DEVICE, "context destroyed before the job finished");
        for (auto &j : pending)
            fail_job_locked(j, VVPT_ERR_DEVICE, "context destroyed before the job started");
        pending.clear();
        completer_stop = true;
        cv_complete.notify_all();
    }
    if (stream)
        cudaStreamSynchronize(stream);
    for (auto &j : running)
        if (j->results)
            cudaFreeAsync(j->results, stream);
}

void Engine::complete_loop()
{
    cudaSetDevice(device);
    for (;;) {
        std::shared_ptr<EJob> j;
        {
            std::unique_lock<std::mutex> lk(m);
            while (completing.empty() && !completer_stop)
                cv_complete.wait(lk);
            if (completing.empty())
                break;
            j = completing.front();
            completing.pop_front();
        }
        cudaError_t e = cudaEventSynchronize(j->done_ev);
        if (e == cudaSuccess && !j->out.on_device && j->staging) {
            const size_t img = (size_t)j->hp.width * j->hp.height * sizeof(float4);
            size_t off = 0;
            for (float *p : {j->out.radiance, j->out.albedo, j->out.normal, j->out.radiance_m2}) {
                if (!p)
                    continue;
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(p, (char *)j->staging + off, img, cudaMemcpyDeviceToHost, copy_stream);
                off += aligned256(img);
            }
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(copy_stream);
        }
        if (j->staging) {
            cudaFreeAsync(j->staging, copy_stream);
            j->staging = nullptr;
        }
        cudaEventDestroy(j->done_ev);
        j->done_ev = nullptr;
        std::lock_guard<std::mutex> lk(m);
        used_bytes -= j->bytes_staging;
        if (e != cudaSuccess) {
            cudaGetLastError();
            fail_job_locked(j, VVPT_ERR_DEVICE, std::string("job completion: ") + cudaGetErrorString(e));
        } else {
            j->state = VVPT_JOB_DONE;
            j->end_ms = now_ms();
            j->scene->jobs_in_flight.fetch_sub(1);
            cv_done.notify_all();
        }
        cv_work.notify_one();
    }
}

void engine_shutdown(vvpt_ctx *ctx)
{
    Engine *eng = nullptr;
    {
        std::lock_guard<std::mutex> lk(ctx->engine_mu);
        eng = ctx->engine;
        ctx->engine = nullptr;
    }
    if (!eng)
        return;
    {
        std::lock_guard<std::mutex> lk(eng->m);
        eng->stop = true;
        eng->cv_work.notify_all();
    }
    eng->worker.join();
    eng->completer.join();
    eng->release_device();
    delete eng;
}

namespace {

vvpt_status get_engine(vvpt_ctx *ctx, Engine **out)
{
    std::lock_guard<std::mutex> lk(ctx->engine_mu);
    if (!ctx->engine) {
        Engine *e = new Engine();
        e->ctx = ctx;
        e->device = ctx->device;
        e->worker = std::thread([e] { e->run(); });
        e->completer = std::thread([e] { e->complete_loop(); });
        ctx->engine = e;
    }
    Engine *e = ctx->engine;
    std::unique_lock<std::mutex> lk2(e->m);
    while (!e->ready)
        e->cv_done.wait(lk2);
    if (e->broken)
        return fail(ctx, VVPT_ERR_DEVICE, e->broken_msg);
    *out = e;
    return VVPT_OK;
}

}  // namespace

}  // namespace vvpt

using namespace vvpt;

extern "C" {

VVPT_API vvpt_status vvpt_submit(vvpt_ctx *ctx, vvpt_scene *scene, const vvpt_scene_data *sd,
                                 const vvpt_render_info *info, const vvpt_outputs *out, vvpt_job *out_job)
{
    if (!ctx || !scene || !sd || !info || !out || !out_job)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    auto j = std::make_shared<EJob>();
    vvpt_status st = make_render_params(ctx, scene, sd, info, j->hp);
    if (st != VVPT_OK)
        return st;
    j->scene = scene;
    j->out = *out;
    j->paths = (uint64_t)j->hp.total_items * j->hp.batch_size;
    if (j->hp.batches && j->hp.depth && j->hp.total_items) {
        j->bytes_results = job_result_bytes(j->hp);
        j->bytes_staging = job_staging_bytes(j->hp, *out);
    }
    Engine *e = nullptr;
    if ((st = get_engine(ctx, &e)) != VVPT_OK)
        return st;
    std::lock_guard<std::mutex> lk(e->m);
    if (e->broken)
        return fail(ctx, VVPT_ERR_DEVICE, e->broken_msg);
    if (ctx->budget_bytes && e->fixed_bytes + j->bytes_results + j->bytes_staging > ctx->budget_bytes)
        return fail(ctx, VVPT_ERR_BUDGET_EXCEEDED,
                    "job needs " + std::to_string(j->bytes_results + j->bytes_staging) +
                        " bytes beside the engine's " + std::to_string(e->fixed_bytes) + "; budget " +
                        std::to_string(ctx->budget_bytes));
    j->id = e->next_id++;
    j->submit_ms = e->now_ms();
    scene->jobs_in_flight.fetch_add(1);
    e->jobs[j->id] = j;
    e->pending.push_back(j);
    e->cv_work.notify_one();
    *out_job = j->id;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_poll(vvpt_ctx *ctx, vvpt_job job, vvpt_job_info *info)
{
    if (!ctx || !info)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    Engine *e = nullptr;
    {
        std::lock_guard<std::mutex> lk(ctx->engine_mu);
        e = ctx->engine;
    }
    if (!e)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "unknown job");
    std::lock_guard<std::mutex> lk(e->m);
    auto it = e->jobs.find(job);
    if (it == e->jobs.end())
        return fail(ctx, VVPT_ERR_INVALID_ARG, "unknown job");
    const EJob &j = *it->second;
    info->state = j.state;
    info->status = j.status;
    info->submit_ms = j.submit_ms;
    info->start_ms = j.start_ms;
    info->end_ms = j.end_ms;
    info->paths = j.paths;
    info->device_bytes = j.bytes_results + j.bytes_staging;
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_wait(vvpt_ctx *ctx, vvpt_job job, double timeout_ms)
{
    if (!ctx)
        return VVPT_ERR_INVALID_ARG;
    Engine *e = nullptr;
    {
        std::lock_guard<std::mutex> lk(ctx->engine_mu);
        e = ctx->engine;
    }
    if (!e)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "unknown job");
    std::unique_lock<std::mutex> lk(e->m);
    auto it = e->jobs.find(job);
    if (it == e->jobs.end())
        return fail(ctx, VVPT_ERR_INVALID_ARG, "unknown job");
    std::shared_ptr<EJob> j = it->second;
    auto finished = [&] { return j->state == VVPT_JOB_DONE || j->state == VVPT_JOB_FAILED; };
    if (timeout_ms < 0)
        e->cv_done.wait(lk, finished);
    else if (!e->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), finished))
        return fail(ctx, VVPT_ERR_TIMEOUT, "job not finished within the timeout");
    if (j->state == VVPT_JOB_FAILED)
        return fail(ctx, j->status, j->error);
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_job_release(vvpt_ctx *ctx, vvpt_job job)
{
    if (!ctx)
        return VVPT_ERR_INVALID_ARG;
    Engine *e = nullptr;
    {
        std::lock_guard<std::mutex> lk(ctx->engine_mu);
        e = ctx->engine;
    }
    if (!e)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "unknown job");
    std::lock_guard<std::mutex> lk(e->m);
    auto it = e->jobs.find(job);
    if (it == e->jobs.end())
        return fail(ctx, VVPT_ERR_INVALID_ARG, "unknown job");
    if (it->second->state != VVPT_JOB_DONE && it->second->state != VVPT_JOB_FAILED)
        return fail(ctx, VVPT_ERR_NOT_READY, "job still queued or running");
    e->jobs.erase(it);
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_set_budget(vvpt_ctx *ctx, uint64_t bytes)
{
    if (!ctx)
        return VVPT_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->engine_mu);
    if (ctx->engine) {
        std::lock_guard<std::mutex> lk2(ctx->engine->m);
        ctx->budget_bytes = bytes;
        ctx->engine->cv_work.notify_one();
    } else {
        ctx->budget_bytes = bytes;
    }
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_engine_stats_get(vvpt_ctx *ctx, vvpt_engine_stats *out)
{
    if (!ctx || !out)
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    Engine *e = nullptr;
    vvpt_status st = get_engine(ctx, &e);
    if (st != VVPT_OK)
        return st;
    std::lock_guard<std::mutex> lk(e->m);
    *out = vvpt_engine_stats{};
    out->fixed_bytes = e->fixed_bytes;
    out->job_bytes = e->used_bytes;
    out->slots = e->slots;
    for (const auto &kv : e->jobs) {
        const uint32_t s = kv.second->state;
        if (s == VVPT_JOB_QUEUED)
            out->queued++;
        else if (s == VVPT_JOB_RUNNING)
            out->running++;
        else
            out->finished++;
    }
    return VVPT_OK;
}

VVPT_API vvpt_status vvpt_render_batch(vvpt_ctx *ctx, uint32_t n, vvpt_scene *const *scenes,
                                       const vvpt_scene_data *sd, const vvpt_render_info *infos,
                                       const vvpt_outputs *outs)
{
    if (!ctx || (n && (!scenes || !sd || !infos || !outs)))
        return fail(ctx, VVPT_ERR_INVALID_ARG, "null argument");
    std::vector<vvpt_job> ids;
    vvpt_status first = VVPT_OK;
    for (uint32_t i = 0; i < n; i++) {
        vvpt_job id = 0;
        vvpt_status st = vvpt_submit(ctx, scenes[i], sd + i, infos + i, outs + i, &id);
        if (st != VVPT_OK) {
            first = st;
            break;
        }
        ids.push_back(id);
    }
    std::string err = first != VVPT_OK ? ctx->last_error : std::string();
    for (vvpt_job id : ids) {
        vvpt_status st = vvpt_wait(ctx, id, -1.0);
        if (st != VVPT_OK && first == VVPT_OK) {
            first = st;
            err = ctx->last_error;
        }
        vvpt_job_release(ctx, id);
    }
    if (first != VVPT_OK)
        return fail(ctx, first, err);
    return VVPT_OK;
}

}  // extern "C"
