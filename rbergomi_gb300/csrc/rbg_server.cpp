// rbg_server.cpp -- a persistent, continuously batched pricing loop.
//
// Calibration traffic sends many independent pricing requests of different
// shapes (N, M, number of strikes, parameters).  The server:
//   * admits requests continuously: a scheduler thread moves submitted
//     requests onto free device slots as soon as a slot and enough of the
//     HBM budget are free (first-in first-out, but a request that does not
//     fit does not block smaller ones behind it).  The footprint charged is
//     M * N * 4 bytes plus the request's tables;
//   * overlaps requests on the device: every slot owns a CUDA stream and its
//     own buffers; small requests (M * N below a threshold) go to
//     high-priority streams, so the hardware scheduler hands them SMs first,
//     and large requests are cut into launches of at most max_batch_paths
//     paths so they yield the GPU between launches;
//   * keeps device-resident Volterra tables (the GEMM strip or the FFT
//     spectrum) cached per (backend, H, N, split), LRU with reference counts;
//   * draws normals from the counter-based Philox stream (seed = the
//     request's seed, counter = path and step), so a request's result does
//     not depend on what else is in flight;
//   * optionally captures each request's device work (everything after the
//     table upload) as a CUDA graph and launches the graph;
//   * records per-request latency (submit -> results on the host).
// Every request runs the mixed form (the tcgen05 Toeplitz GEMM, N <= 4096).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "rbg_internal.hpp"
#include "rbg_mixed.hpp"

namespace rbg {

namespace {

using Clock = std::chrono::steady_clock;

// Stream-ordered, grow-only device buffer from the server's memory pool.
struct SBuf {
    void* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t bytes, cudaStream_t st, cudaMemPool_t pool)
    {
        if (bytes <= n) return cudaSuccess;
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        n = 0;
        const size_t want = std::max(bytes, (size_t)4096);
        cudaError_t e = cudaMallocFromPoolAsync(&p, want, pool, st);
        if (e == cudaSuccess) n = want;
        return e;
    }
};

// Outputs the pinned result buffer of every slot holds from the start: a
// slot that had to grow it would call cudaFreeHost, which waits for the
// whole device (every request in flight) on the scheduler thread.
constexpr size_t kPinOutputs = 4096;
// A shared launch prices at most this many outputs (all its requests' together)
// and this many requests.
constexpr int kBatchOutputs = (int)kPinOutputs;
constexpr int kBatchJobsMax = 64;
// Completion polling interval while work is in flight: on average half of it
// is added to every request's latency.
#ifndef RBG_SERVER_POLL_US
#define RBG_SERVER_POLL_US 10
#endif
constexpr int kPollUs = RBG_SERVER_POLL_US;

struct Req {
    uint64_t id = 0;
    Plan plan;
    rbg_options opt{};
    int64_t M = 0;
    MixedJob job;
    std::vector<OutDev> outs;
    std::vector<double> Tv;
    size_t footprint = 0;
    double work = 0;  // path-steps
    std::vector<double> res;
    int status = RBG_OK;
    std::string err;
    bool done = false;
    std::vector<int> cache_keys;  // cache entries pinned while in flight
    bool batchable = false;       // priced in shared launches (one one-pass launch, RT)
    Clock::time_point t_submit, t_start, t_launched, t_done;
};

// A shared launch in flight: the requests it prices, where each one's
// results sit in the pinned buffer, and its buffers (grow-only; results at a
// fixed capacity so that its CUDA graph keeps one shape).
struct BatchSlot {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    SBuf in, ivb, part, acc, res;
    double* pin = nullptr;  // [0] error word, then 5 * kBatchOutputs results
    std::vector<Req*> reqs;
    std::vector<size_t> res_off;  // doubles, per request
    std::vector<unsigned char> host_in, host_tab;
    cudaGraphExec_t graph = nullptr;
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    bool high = false;
    SBuf ws, ivb, part, acc, res, outs;
    double* pin = nullptr;  // [0] error word, then 5 * n_out results
    size_t pin_n = 0;
    Req* req = nullptr;
    // graph cache: one instantiated graph per launch shape
    std::map<std::string, cudaGraphExec_t> graphs;
};

struct CacheEntry {
    void* dev = nullptr;
    size_t bytes = 0;
    int refs = 0;
    cudaEvent_t ready = nullptr;
    std::list<int>::iterator lru;
};

}  // namespace

struct Server {
    rbg_server_config cfg{};
    int dev = 0;
    std::vector<Slot> slots;
    std::vector<BatchSlot> bslots;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req*> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Req>> reqs;
    uint64_t next_id = 1;
    size_t in_use = 0;
    bool stop = false;
    std::thread thr;
    cudaStream_t copy_st = nullptr;
    // device memory of slots and tables: a pool that keeps freed memory
    // mapped (release threshold = all), so growing a buffer or replacing a
    // table does not map new pages on the scheduler's path
    cudaMemPool_t pool = nullptr;
    // table cache
    std::map<std::tuple<int, uint64_t, int, int>, int> cache_index;
    std::vector<CacheEntry> cache;
    std::list<int> lru;
    // statistics
    uint64_t completed = 0, failed = 0, cache_hits = 0, cache_misses = 0, graph_launches = 0;
    uint64_t graph_instantiations = 0, graph_updates = 0, max_launch_us = 0, pin_growths = 0;
    uint64_t batches = 0, batched_requests = 0;
    // longest scheduler-thread time per launch phase (us): buffers, tables, uploads, graph
    uint64_t max_alloc_us = 0, max_tables_us = 0, max_upload_us = 0, max_graph_us = 0;
    double busy_since_ms = -1;

    void run();
    int launch(Slot& s, Req& r, std::string& err);
    void finish(Slot& s);
    int launch_batch(BatchSlot& b, std::vector<Req*>& rs, std::string& err);
    void finish_batch(BatchSlot& b, cudaError_t q);
    int graph_run(cudaGraphExec_t& exec, cudaGraph_t g, cudaStream_t st, std::string& err);
    void fail_request(Req* r, int status, const std::string& err);
    int acquire_tables(Req& r, cudaStream_t st, std::string& err);
    void release_tables(Req& r);
};

// Times the phases of one launch on the scheduler thread into the server's maxima.
struct Laps {
    Clock::time_point t = Clock::now();
    void lap(uint64_t& mx)
    {
        const Clock::time_point n = Clock::now();
        mx = std::max<uint64_t>(mx, (uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(n - t).count());
        t = n;
    }
};

static uint64_t hbits(double x)
{
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
}

int Server::acquire_tables(Req& r, cudaStream_t st, std::string& err)
{
    MixedJob& job = r.job;
    job.table_dev.assign(job.launches.size(), nullptr);
    for (size_t i = 0; i < job.launches.size(); ++i) {
        const MixedArgs& A = job.launches[i].args;
        const double H = r.plan.vols[r.plan.vgs[A.g0].vol].H;
        auto key = std::make_tuple(job.backend, hbits(H), r.plan.N, job.split);
        size_t off = 0, bytes = 0;
        mixed_table_range(job, (int)i, &off, &bytes);
        int idx;
        auto it = cache_index.find(key);
        if (it != cache_index.end()) {
            idx = it->second;
            lru.erase(cache[idx].lru);
            ++cache_hits;
        } else {
            ++cache_misses;
            // evict unreferenced entries beyond the capacity
            while ((int)cache_index.size() >= cfg.table_cache_entries) {
                auto victim = std::find_if(lru.rbegin(), lru.rend(), [&](int k) { return cache[k].refs == 0; });
                if (victim == lru.rend()) break;
                const int k = *victim;
                for (auto jt = cache_index.begin(); jt != cache_index.end(); ++jt)
                    if (jt->second == k) { cache_index.erase(jt); break; }
                lru.erase(std::next(victim).base());
                cudaFreeAsync(cache[k].dev, copy_st);
                cache[k].dev = nullptr;
            }
            idx = -1;
            for (size_t k = 0; k < cache.size(); ++k)
                if (!cache[k].dev && cache[k].refs == 0) { idx = (int)k; break; }
            if (idx < 0) {
                cache.emplace_back();
                idx = (int)cache.size() - 1;
                cudaEventCreateWithFlags(&cache[idx].ready, cudaEventDisableTiming);
            }
            CacheEntry& e = cache[idx];
            cudaError_t ce = cudaMallocFromPoolAsync(&e.dev, bytes, pool, copy_st);
            if (ce == cudaSuccess)
                ce = cudaMemcpyAsync(e.dev, job.host_ws.data() + off, bytes, cudaMemcpyHostToDevice, copy_st);
            if (ce == cudaSuccess) ce = cudaEventRecord(e.ready, copy_st);
            if (ce != cudaSuccess) {
                cudaGetLastError();
                err = std::string("table cache: ") + cudaGetErrorString(ce);
                return RBG_ERR_CUDA;
            }
            // the copy reads host_ws: finish it before the request (and its host image) can go
            cudaStreamSynchronize(copy_st);
            e.bytes = bytes;
            cache_index[key] = idx;
        }
        CacheEntry& e = cache[idx];
        lru.push_front(idx);
        e.lru = lru.begin();
        ++e.refs;
        r.cache_keys.push_back(idx);
        cudaStreamWaitEvent(st, e.ready, 0);
        job.table_dev[i] = e.dev;
    }
    return RBG_OK;
}

void Server::release_tables(Req& r)
{
    for (int k : r.cache_keys) --cache[k].refs;
    r.cache_keys.clear();
}

int Server::launch(Slot& s, Req& r, std::string& err)
{
    cudaStream_t st = s.st;
    MixedJob& job = r.job;
    const int no = (int)r.plan.outs.size();
    const int64_t B = job.batch;
    const int G = payoff_paths_per_thread(B, job.sms);
    const int64_t rows = job.fused ? mixed_part_rows(job, B) : (B + 256 * (int64_t)G - 1) / (256 * (int64_t)G);
    Laps laps;
    cudaError_t e = s.ws.ensure(job.workspace_bytes, st, pool);
    if (e == cudaSuccess && !job.fused)
        e = s.ivb.ensure(sizeof(float) * 2 * r.plan.vgs.size() * (size_t)B, st, pool);
    if (e == cudaSuccess) e = s.part.ensure(sizeof(double) * 4 * no * (size_t)rows, st, pool);
    if (e == cudaSuccess) e = s.acc.ensure(sizeof(double) * 4 * no, st, pool);
    if (e == cudaSuccess) e = s.res.ensure(sizeof(double) * 5 * no, st, pool);
    if (e == cudaSuccess) e = s.outs.ensure(sizeof(OutDev) * no + sizeof(double) * no + 256, st, pool);
    const size_t pin_need = sizeof(double) * (1 + 5 * (size_t)no);
    if (e == cudaSuccess && s.pin_n < pin_need) {
        // beyond kPinOutputs outputs only: cudaFreeHost waits for the device
        ++pin_growths;
        if (s.pin) cudaFreeHost(s.pin);
        s.pin = nullptr;
        s.pin_n = 0;
        e = cudaMallocHost((void**)&s.pin, pin_need);
        if (e == cudaSuccess) s.pin_n = pin_need;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("slot buffers: ") + cudaGetErrorString(e);
        return RBG_ERR_NOMEM;
    }
    laps.lap(max_alloc_us);
    int rc = acquire_tables(r, st, err);
    if (rc) return rc;
    laps.lap(max_tables_us);
    OutDev* d_outs = (OutDev*)s.outs.p;
    double* d_T = (double*)((unsigned char*)s.outs.p + ((sizeof(OutDev) * no + 255) / 256) * 256);
    // inputs (pageable host memory; the request keeps them alive until it completes)
    e = cudaMemcpyAsync(s.ws.p, job.host_ws.data(), job.host_ws.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_outs, r.outs.data(), sizeof(OutDev) * no, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_T, r.Tv.data(), sizeof(double) * no, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("request upload: ") + cudaGetErrorString(e);
        return RBG_ERR_CUDA;
    }

    laps.lap(max_upload_us);
    // device work of the request: captured as a CUDA graph when configured, for
    // requests of one launch (replaying a many-launch request saves nothing
    // measurable, and instantiating its graph took milliseconds)
    const bool graph = cfg.use_graphs != 0 && r.M <= B;
    if (graph) {
        e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaGetLastError();
            err = std::string("graph capture: ") + cudaGetErrorString(e);
            return RBG_ERR_CUDA;
        }
    }
    std::string kerr;
    rc = RBG_OK;
    cudaMemsetAsync(s.acc.p, 0, sizeof(double) * 4 * no, st);
    for (int64_t m0 = 0; m0 < r.M && rc == RBG_OK; m0 += B) {
        const int64_t b = std::min(B, r.M - m0);
        if (job.fused) {
            const int nr = mixed_part_rows(job, b);
            cudaMemsetAsync(s.part.p, 0, sizeof(double) * 4 * no * (size_t)nr, st);
            rc = mixed_launch(job, s.ws.p, r.opt.seed, r.opt.path_offset + m0, b, nullptr, st, kerr, nullptr,
                              nullptr, (double*)s.part.p);
            if (rc == RBG_OK) launch_accumulate((const double*)s.part.p, nr, no, (double*)s.acc.p, st);
        } else {
            rc = mixed_launch(job, s.ws.p, r.opt.seed, r.opt.path_offset + m0, b, s.ivb.p, st, kerr);
            const int nchunks = (int)((b + 256 * (int64_t)G - 1) / (256 * (int64_t)G));
            if (rc == RBG_OK) {
                launch_payoff_sums_f32(d_outs, no, s.ivb.p, b, G, (double*)s.part.p, nchunks, st);
                launch_accumulate((const double*)s.part.p, nchunks, no, (double*)s.acc.p, st);
            }
        }
    }
    if (rc == RBG_OK) {
        launch_finalize((const double*)s.acc.p, no, r.M, d_outs, d_T, r.opt.compute_iv, (double*)s.res.p, st);
        cudaMemcpyAsync(s.pin, (unsigned char*)s.ws.p + job.off_err, 4, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(s.pin + 1, s.res.p, sizeof(double) * 5 * no, cudaMemcpyDeviceToHost, st);
    }
    if (graph) {
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(st, &g);
        if (rc == RBG_OK && e == cudaSuccess) {
            // one executable graph per launch shape, updated in place for new parameters
            // keyed by the graph's topology and node shapes (kernel variant, launches
            // per batch, batches, outputs): requests of other M, N or parameters
            // with the same key update the executable graph in place
            char key[128];
            const MixedArgs& A0 = job.launches[0].args;
            std::snprintf(key, sizeof key, "%d/%d/%d/%d/%lld/%d/%d", job.backend, A0.n0 > 0 ? 1 : 0, A0.logL,
                          (int)job.launches.size(), (long long)((r.M + B - 1) / B), no, job.fused ? 1 : 0);
            auto it = s.graphs.find(key);
            bool ok = false;
            if (it != s.graphs.end()) {
                cudaGraphExecUpdateResultInfo info;
                ok = cudaGraphExecUpdate(it->second, g, &info) == cudaSuccess;
                if (ok) ++graph_updates;
                if (!ok) {
                    cudaGetLastError();
                    cudaGraphExecDestroy(it->second);
                    s.graphs.erase(it);
                }
            }
            if (!ok) {
                cudaGraphExec_t ex = nullptr;
                e = cudaGraphInstantiate(&ex, g, 0);
                if (e == cudaSuccess) {
                    s.graphs[key] = ex;
                    ok = true;
                    ++graph_instantiations;
                }
            }
            if (ok) {
                e = cudaGraphLaunch(s.graphs[key], st);
                ++graph_launches;
            }
        }
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess && rc == RBG_OK) {
            cudaGetLastError();
            err = std::string("graph launch: ") + cudaGetErrorString(e);
            return RBG_ERR_CUDA;
        }
    }
    laps.lap(max_graph_us);
    if (rc != RBG_OK) {
        err = kerr;
        return rc;
    }
    e = cudaEventRecord(s.ev, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("request launch: ") + cudaGetErrorString(e);
        return RBG_ERR_CUDA;
    }
    return RBG_OK;
}

void Server::finish(Slot& s)
{
    Req& r = *s.req;
    const int no = (int)r.plan.outs.size();
    unsigned int word = 0;
    std::memcpy(&word, s.pin, 4);
    if (word != 0) {
        r.status = RBG_ERR_TIMEOUT;
        r.err = "mixed kernel: a bounded pipeline wait expired (site " + std::to_string(word) + ")";
    } else {
        r.res.assign(s.pin + 1, s.pin + 1 + 5 * (size_t)no);
    }
    r.t_done = Clock::now();
    r.done = true;
    release_tables(r);
    in_use -= r.footprint;
    if (r.status == RBG_OK) ++completed; else ++failed;
    s.req = nullptr;
}

void Server::fail_request(Req* r, int status, const std::string& err)
{
    r->status = status;
    r->err = err;
    r->t_done = Clock::now();
    r->done = true;
    release_tables(*r);
    in_use -= r->footprint;
    ++failed;
}

// Updates `exec` in place from the captured graph, or instantiates it anew,
// and launches it.
int Server::graph_run(cudaGraphExec_t& exec, cudaGraph_t g, cudaStream_t st, std::string& err)
{
    bool ok = false;
    if (exec) {
        cudaGraphExecUpdateResultInfo info;
        ok = cudaGraphExecUpdate(exec, g, &info) == cudaSuccess;
        if (ok) {
            ++graph_updates;
        } else {
            cudaGetLastError();
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
    }
    cudaError_t e = cudaSuccess;
    if (!ok) {
        e = cudaGraphInstantiate(&exec, g, 0);
        if (e == cudaSuccess) ++graph_instantiations;
        else exec = nullptr;
    }
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("graph launch: ") + cudaGetErrorString(e);
        return RBG_ERR_CUDA;
    }
    ++graph_launches;
    return RBG_OK;
}

// One shared launch for requests rs (all batchable, one split): their
// workspace images, output tables and the job tables go up in one copy;
// then the job-table path, payoff, merge and finalize kernels and the
// result copy run on the batch slot's stream, as one CUDA graph.
int Server::launch_batch(BatchSlot& b, std::vector<Req*>& rs, std::string& err)
{
    cudaStream_t st = b.st;
    const int n = (int)rs.size();
    Laps laps;
    for (Req* r : rs) {
        const int rc = acquire_tables(*r, st, err);
        if (rc) return rc;
    }
    laps.lap(max_tables_us);
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    std::vector<size_t> o_ws(n), o_outs(n), o_T(n), o_ivb(n), o_part(n), o_acc(n), o_res(n);
    std::vector<int> G(n), nch(n);
    size_t in_bytes = 256, ivb_bytes = 0, part_bytes = 0, acc_bytes = 0, res_d = 0;
    for (int k = 0; k < n; ++k) {
        const Req& r = *rs[k];
        const int no = (int)r.plan.outs.size();
        const int64_t B = r.M;  // one launch: the request's whole path count
        o_ws[k] = in_bytes;
        in_bytes = up(in_bytes + r.job.host_ws.size());
        o_outs[k] = in_bytes;
        in_bytes = up(in_bytes + sizeof(OutDev) * no);
        o_T[k] = in_bytes;
        in_bytes = up(in_bytes + sizeof(double) * no);
        o_ivb[k] = ivb_bytes;
        ivb_bytes = up(ivb_bytes + sizeof(float) * 2 * r.plan.vgs.size() * (size_t)B);
        G[k] = payoff_paths_per_thread(r.job.batch, r.job.sms);
        nch[k] = (int)((B + 256 * (int64_t)G[k] - 1) / (256 * (int64_t)G[k]));
        o_part[k] = part_bytes;
        part_bytes = up(part_bytes + sizeof(double) * 4 * no * (size_t)nch[k]);
        o_acc[k] = acc_bytes;
        acc_bytes = up(acc_bytes + sizeof(double) * 4 * no);
        o_res[k] = res_d;
        res_d += 5 * (size_t)no;
    }
    const size_t off_tab = in_bytes;
    in_bytes = up(in_bytes + mixed_jobs_table_bytes(n));
    const size_t off_pj = in_bytes;
    in_bytes = up(in_bytes + sizeof(PayoffJob) * n);
    const size_t off_aj = in_bytes;
    in_bytes = up(in_bytes + sizeof(AccJob) * n);
    const size_t off_fj = in_bytes;
    in_bytes = up(in_bytes + sizeof(FinJob) * n);
    cudaError_t e = b.in.ensure(in_bytes, st, pool);
    if (e == cudaSuccess) e = b.ivb.ensure(ivb_bytes, st, pool);
    if (e == cudaSuccess) e = b.part.ensure(part_bytes, st, pool);
    if (e == cudaSuccess) e = b.acc.ensure(acc_bytes, st, pool);
    if (e == cudaSuccess) e = b.res.ensure(sizeof(double) * 5 * kBatchOutputs, st, pool);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("batch buffers: ") + cudaGetErrorString(e);
        return RBG_ERR_NOMEM;
    }
    laps.lap(max_alloc_us);
    unsigned char* din = (unsigned char*)b.in.p;
    unsigned char* divb = (unsigned char*)b.ivb.p;
    unsigned char* dpart = (unsigned char*)b.part.p;
    unsigned char* dacc = (unsigned char*)b.acc.p;
    double* dres = (double*)b.res.p;
    b.host_in.assign(in_bytes, 0);  // error word at 0 cleared with the upload
    std::vector<MixedJobRef> refs(n);
    PayoffJob* pj = (PayoffJob*)(b.host_in.data() + off_pj);
    AccJob* aj = (AccJob*)(b.host_in.data() + off_aj);
    FinJob* fj = (FinJob*)(b.host_in.data() + off_fj);
    int64_t pblocks = 0, ablocks = 0;
    for (int k = 0; k < n; ++k) {
        Req& r = *rs[k];
        const int no = (int)r.plan.outs.size();
        std::memcpy(b.host_in.data() + o_ws[k], r.job.host_ws.data(), r.job.host_ws.size());
        std::memcpy(b.host_in.data() + o_outs[k], r.outs.data(), sizeof(OutDev) * no);
        std::memcpy(b.host_in.data() + o_T[k], r.Tv.data(), sizeof(double) * no);
        refs[k] = MixedJobRef{&r.job, din + o_ws[k], r.opt.seed, r.opt.path_offset, r.M, divb + o_ivb[k]};
        const OutDev* outs = (const OutDev*)(din + o_outs[k]);
        double* acc = (double*)(dacc + o_acc[k]);
        pj[k] = PayoffJob{outs, (const float2*)(divb + o_ivb[k]), (double*)(dpart + o_part[k]), r.M, pblocks, no, G[k],
                          nch[k], 0};
        pblocks += (int64_t)nch[k] * ((no + 7) / 8);
        aj[k] = AccJob{(const double*)(dpart + o_part[k]), acc, ablocks, nch[k], no};
        fj[k] = FinJob{acc, outs, (const double*)(din + o_T[k]), dres + o_res[k], r.M, ablocks, no, r.opt.compute_iv};
        ablocks += no;
    }
    MixedArgs LA;
    const int grid = mixed_jobs_prepare(refs, din + off_tab, (unsigned int*)din, rs[0]->job.sms, b.host_tab, &LA, err);
    if (grid < 1) return RBG_ERR_ARG;
    std::memcpy(b.host_in.data() + off_tab, b.host_tab.data(), b.host_tab.size());
    // pageable source: staged before the call returns, so host_in may be reused
    e = cudaMemcpyAsync(din, b.host_in.data(), in_bytes, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("batch upload: ") + cudaGetErrorString(e);
        return RBG_ERR_CUDA;
    }
    laps.lap(max_upload_us);
    const bool graph = cfg.use_graphs != 0;
    if (graph && (e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        cudaGetLastError();
        err = std::string("graph capture: ") + cudaGetErrorString(e);
        return RBG_ERR_CUDA;
    }
    int rc = mixed_launch_jobs(LA, rs[0]->job.split, grid, st, err);
    if (rc == RBG_OK) {
        launch_payoff_sums_f32_jobs((const PayoffJob*)(din + off_pj), n, pblocks, st);
        launch_accumulate_jobs((const AccJob*)(din + off_aj), n, ablocks, st);
        launch_finalize_jobs((const FinJob*)(din + off_fj), n, ablocks, st);
        cudaMemcpyAsync(b.pin, din, 4, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(b.pin + 1, dres, sizeof(double) * 5 * kBatchOutputs, cudaMemcpyDeviceToHost, st);
    }
    if (graph) {
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(st, &g);
        if (rc == RBG_OK && e == cudaSuccess) rc = graph_run(b.graph, g, st, err);
        else if (rc == RBG_OK) {
            cudaGetLastError();
            err = std::string("graph capture: ") + cudaGetErrorString(e);
            rc = RBG_ERR_CUDA;
        }
        if (g) cudaGraphDestroy(g);
    }
    laps.lap(max_graph_us);
    if (rc != RBG_OK) return rc;
    if ((e = cudaEventRecord(b.ev, st)) != cudaSuccess) {
        cudaGetLastError();
        err = std::string("batch launch: ") + cudaGetErrorString(e);
        return RBG_ERR_CUDA;
    }
    b.reqs = rs;
    b.res_off = o_res;
    ++batches;
    batched_requests += (uint64_t)n;
    return RBG_OK;
}

void Server::finish_batch(BatchSlot& b, cudaError_t q)
{
    unsigned int word = 0;
    std::memcpy(&word, b.pin, 4);
    for (size_t k = 0; k < b.reqs.size(); ++k) {
        Req* r = b.reqs[k];
        if (q != cudaSuccess) {
            fail_request(r, RBG_ERR_CUDA, std::string("device: ") + cudaGetErrorString(q));
            continue;
        }
        if (word != 0) {
            fail_request(r, RBG_ERR_TIMEOUT, "mixed kernel: a bounded pipeline wait expired (site " +
                                                 std::to_string(word) + ")");
            continue;
        }
        const size_t no = r->plan.outs.size();
        r->res.assign(b.pin + 1 + b.res_off[k], b.pin + 1 + b.res_off[k] + 5 * no);
        r->t_done = Clock::now();
        r->done = true;
        release_tables(*r);
        in_use -= r->footprint;
        ++completed;
    }
    b.reqs.clear();
}

void Server::run()
{
    cudaSetDevice(dev);
    std::unique_lock<std::mutex> lk(mu);
    while (true) {
        bool progressed = false;
        // completions
        for (Slot& s : slots) {
            if (!s.req) continue;
            cudaError_t q = cudaEventQuery(s.ev);
            if (q == cudaSuccess) {
                finish(s);
                progressed = true;
            } else if (q != cudaErrorNotReady) {
                cudaGetLastError();
                s.req->status = RBG_ERR_CUDA;
                s.req->err = std::string("device: ") + cudaGetErrorString(q);
                s.req->t_done = Clock::now();
                s.req->done = true;
                release_tables(*s.req);
                in_use -= s.req->footprint;
                ++failed;
                s.req = nullptr;
                progressed = true;
            }
        }
        for (BatchSlot& b : bslots) {
            if (b.reqs.empty()) continue;
            const cudaError_t q = cudaEventQuery(b.ev);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) cudaGetLastError();
            finish_batch(b, q);
            progressed = true;
        }
        if (progressed) cv_done.notify_all();
        auto busy_now = [&] {
            for (Slot& s : slots)
                if (s.req) return true;
            for (BatchSlot& b : bslots)
                if (!b.reqs.empty()) return true;
            return false;
        };
        if (stop && pending.empty() && !busy_now()) break;
        // shared launches: every free batch slot takes the batchable requests
        // pending now, in arrival order, up to its job / output / work limits --
        // after the batching window, when one is set and fewer than a full
        // batch are pending
        Clock::time_point wake = Clock::time_point::max();
        if (cfg.batch_wait_us > 0 && !stop) {
            int nb = 0;
            Clock::time_point oldest = Clock::time_point::max();
            for (Req* r : pending)
                if (r->batchable) {
                    ++nb;
                    oldest = std::min(oldest, r->t_submit);
                }
            const auto window = std::chrono::duration_cast<Clock::duration>(
                std::chrono::duration<double, std::micro>(cfg.batch_wait_us));
            if (nb > 0 && nb < cfg.max_batch_jobs && Clock::now() < oldest + window) wake = oldest + window;
        }
        for (BatchSlot& b : bslots) {
            if (wake != Clock::time_point::max()) break;  // inside the batching window
            if (!b.reqs.empty()) continue;
            std::vector<Req*> batch;
            int split = -1, outs = 0;
            double work = 0;
            size_t fp = 0;
            for (auto it = pending.begin(); it != pending.end() && (int)batch.size() < cfg.max_batch_jobs;) {
                Req* r = *it;
                const int no = (int)r->plan.outs.size();
                const bool take = r->batchable && (split < 0 || r->job.split == split) &&
                                  outs + no <= kBatchOutputs &&
                                  (batch.empty() || work + r->work <= cfg.batch_path_steps) &&
                                  (in_use + fp + r->footprint <= cfg.hbm_budget || (in_use == 0 && batch.empty()));
                if (!take) {
                    ++it;
                    continue;
                }
                split = r->job.split;
                outs += no;
                work += r->work;
                fp += r->footprint;
                batch.push_back(r);
                it = pending.erase(it);
            }
            if (batch.empty()) break;
            in_use += fp;
            const Clock::time_point t0 = Clock::now();
            for (Req* r : batch) r->t_start = t0;
            std::string err;
            const int rc = launch_batch(b, batch, err);
            const Clock::time_point t1 = Clock::now();
            max_launch_us = std::max<uint64_t>(
                max_launch_us, (uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count());
            for (Req* r : batch) r->t_launched = t1;
            if (rc != RBG_OK) {
                for (Req* r : batch) fail_request(r, rc, err);
                cv_done.notify_all();
            }
            progressed = true;
        }
        // admissions: first fit in arrival order
        for (auto it = pending.begin(); it != pending.end();) {
            Req* r = *it;
            if (r->batchable && !bslots.empty()) {  // waits for a batch slot
                ++it;
                continue;
            }
            const bool small = r->work <= cfg.small_request_path_steps;
            Slot* free_slot = nullptr;
            for (Slot& s : slots)
                if (!s.req && (s.high == small || (!small && s.high == false))) { free_slot = &s; break; }
            if (!free_slot && small)
                for (Slot& s : slots)
                    if (!s.req) { free_slot = &s; break; }
            const bool fits = in_use + r->footprint <= cfg.hbm_budget || in_use == 0;
            if (!free_slot || !fits) {
                ++it;
                continue;
            }
            it = pending.erase(it);
            free_slot->req = r;
            in_use += r->footprint;
            r->t_start = Clock::now();
            std::string err;
            const int rc = launch(*free_slot, *r, err);
            r->t_launched = Clock::now();
            max_launch_us = std::max<uint64_t>(
                max_launch_us,
                (uint64_t)std::chrono::duration_cast<std::chrono::microseconds>(r->t_launched - r->t_start).count());
            if (rc != RBG_OK) {
                r->status = rc;
                r->err = err;
                r->t_done = Clock::now();
                r->done = true;
                release_tables(*r);
                in_use -= r->footprint;
                ++failed;
                free_slot->req = nullptr;
                cv_done.notify_all();
            }
            progressed = true;
        }
        if (!progressed) {
            // poll the device quickly while work is in flight, sleep otherwise (until
            // the batching window closes, at the latest)
            Clock::duration d = busy_now() ? Clock::duration(std::chrono::microseconds(kPollUs))
                                           : Clock::duration(std::chrono::milliseconds(5));
            if (wake != Clock::time_point::max()) d = std::min(d, std::max(Clock::duration(0), wake - Clock::now()));
            cv_work.wait_for(lk, d);
        }
    }
}

}  // namespace rbg

using namespace rbg;

struct rbg_server {
    std::unique_ptr<Server> s;
};

static thread_local std::string g_srv_err;

static int srv_fail(int code, const std::string& m)
{
    g_srv_err = m;
    return code;
}

extern "C" {

void rbg_server_default_config(rbg_server_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->slots = 12;
    c->high_priority_slots = 8;
    c->hbm_budget = (uint64_t)96 << 30;
    c->max_batch_paths = (int64_t)1 << 19;
    c->small_request_path_steps = (double)(1u << 28);
    c->table_cache_entries = 256;
    c->use_graphs = 1;
    c->device = -1;
    c->batch_slots = 8;
    c->max_batch_jobs = kBatchJobsMax;
    c->batch_path_steps = (double)(1u << 30);
    c->batch_wait_us = 0.0;
}

const char* rbg_server_last_error(void) { return g_srv_err.c_str(); }

int rbg_server_create(const rbg_server_config* cfg_in, rbg_server** out)
{
    if (!out) return srv_fail(RBG_ERR_ARG, "null output");
    rbg_server_config cfg;
    rbg_server_default_config(&cfg);
    if (cfg_in) cfg = *cfg_in;
    if (cfg.slots < 1 || cfg.slots > 64 || cfg.high_priority_slots < 0 || cfg.high_priority_slots > cfg.slots)
        return srv_fail(RBG_ERR_ARG, "slots must be 1..64 and high_priority_slots <= slots");
    if (cfg.batch_slots < 0 || cfg.batch_slots > 16 || cfg.max_batch_jobs < 1 || cfg.max_batch_jobs > kBatchJobsMax)
        return srv_fail(RBG_ERR_ARG, "batch_slots must be 0..16 and max_batch_jobs 1..64");
    std::unique_ptr<Server> s(new Server());
    s->cfg = cfg;
    int dev = cfg.device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return srv_fail(RBG_ERR_CUDA, "no CUDA device");
    s->dev = dev;
    if (cudaSetDevice(dev) != cudaSuccess) return srv_fail(RBG_ERR_CUDA, "cudaSetDevice failed");
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    s->slots.resize(cfg.slots);
    for (int i = 0; i < cfg.slots; ++i) {
        Slot& sl = s->slots[i];
        sl.high = i < cfg.high_priority_slots;
        if (cudaStreamCreateWithPriority(&sl.st, cudaStreamNonBlocking, sl.high ? hi : lo) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess)
            return srv_fail(RBG_ERR_CUDA, "stream/event creation failed");
    }
    if (cudaStreamCreateWithFlags(&s->copy_st, cudaStreamNonBlocking) != cudaSuccess)
        return srv_fail(RBG_ERR_CUDA, "stream creation failed");
    cudaMemPoolProps pp;
    std::memset(&pp, 0, sizeof pp);
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = dev;
    uint64_t keep = ~(uint64_t)0;
    if (cudaMemPoolCreate(&s->pool, &pp) != cudaSuccess ||
        cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
        cudaGetLastError();
        return srv_fail(RBG_ERR_CUDA, "memory pool creation failed");
    }
    for (Slot& sl : s->slots) {
        const size_t bytes = sizeof(double) * (1 + 5 * kPinOutputs);
        if (cudaMallocHost((void**)&sl.pin, bytes) != cudaSuccess) {
            cudaGetLastError();
            return srv_fail(RBG_ERR_NOMEM, "pinned result buffers");
        }
        sl.pin_n = bytes;
    }
    s->bslots.resize(cfg.batch_slots);
    for (BatchSlot& b : s->bslots) {
        if (cudaStreamCreateWithPriority(&b.st, cudaStreamNonBlocking, hi) != cudaSuccess ||
            cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming) != cudaSuccess ||
            cudaMallocHost((void**)&b.pin, sizeof(double) * (1 + 5 * (size_t)kBatchOutputs)) != cudaSuccess) {
            cudaGetLastError();
            return srv_fail(RBG_ERR_CUDA, "batch slot creation failed");
        }
    }
    // every kernel the loop may launch, loaded now rather than mid-stream
    mixed_preload();
    reduce_preload();
    Server* raw = s.get();
    s->thr = std::thread([raw] { raw->run(); });
    *out = new rbg_server{std::move(s)};
    return RBG_OK;
}

int rbg_server_submit(rbg_server* srv, const rbg_params* p, const rbg_options* o, uint64_t* ticket)
{
    if (!srv || !p || !ticket) return srv_fail(RBG_ERR_ARG, "null argument");
    std::unique_ptr<Req> r(new Req());
    r->t_submit = Clock::now();
    std::string err;
    if (!build_plan(*p, r->plan, err)) return srv_fail(RBG_ERR_ARG, err);
    rbg_default_options(&r->opt);
    if (o) r->opt = *o;
    r->opt.precision = RBG_MIXED;
    r->opt.stream = nullptr;
    r->M = p->M;
    cudaSetDevice(srv->s->dev);
    int rc = mixed_prepare(r->plan, r->opt, p->M, r->job, err, srv->s->cfg.max_batch_paths);
    if (rc) return srv_fail(rc, err);
    const int no = (int)r->plan.outs.size();
    r->outs.resize(no);
    r->Tv.resize(no);
    for (int i = 0; i < no; ++i) {
        r->outs[i] = OutDev{r->plan.outs[i].rho, r->plan.outs[i].K, r->plan.outs[i].vg, 0};
        r->Tv[i] = r->plan.outs[i].T;
    }
    r->work = (double)p->M * p->N * (double)r->plan.vols.size();
    r->batchable = srv->s->cfg.batch_slots > 0 && mixed_job_batchable(r->job) && r->M <= r->job.batch &&
                   no <= kBatchOutputs;
    r->footprint = (size_t)p->M * (size_t)p->N * 4 + r->job.workspace_bytes;
    Server& s = *srv->s;
    {
        std::lock_guard<std::mutex> lk(s.mu);
        if (s.stop) return srv_fail(RBG_ERR_ARG, "server is stopping");
        r->id = s.next_id++;
        *ticket = r->id;
        s.pending.push_back(r.get());
        s.reqs[r->id] = std::move(r);
    }
    s.cv_work.notify_one();
    return RBG_OK;
}

int rbg_server_poll(rbg_server* srv, uint64_t ticket, int* done)
{
    if (!srv || !done) return srv_fail(RBG_ERR_ARG, "null argument");
    Server& s = *srv->s;
    std::lock_guard<std::mutex> lk(s.mu);
    auto it = s.reqs.find(ticket);
    if (it == s.reqs.end()) return srv_fail(RBG_ERR_ARG, "unknown ticket");
    *done = it->second->done ? 1 : 0;
    return RBG_OK;
}

int rbg_server_wait(rbg_server* srv, uint64_t ticket, double* price, double* stat, double* iv, double* latency_ms)
{
    double t[3];
    const int rc = rbg_server_wait_timed(srv, ticket, price, stat, iv, t);
    if (latency_ms) *latency_ms = t[2];
    return rc;
}

int rbg_server_wait_timed(rbg_server* srv, uint64_t ticket, double* price, double* stat, double* iv, double* times)
{
    if (!srv) return srv_fail(RBG_ERR_ARG, "null server");
    Server& s = *srv->s;
    std::unique_lock<std::mutex> lk(s.mu);
    auto it = s.reqs.find(ticket);
    if (it == s.reqs.end()) return srv_fail(RBG_ERR_ARG, "unknown ticket");
    Req* r = it->second.get();
    s.cv_done.wait(lk, [&] { return r->done; });
    const int status = r->status;
    if (status == RBG_OK) {
        const size_t no = r->plan.outs.size();
        if (price) std::memcpy(price, r->res.data(), no * sizeof(double));
        if (stat) std::memcpy(stat, r->res.data() + no, no * sizeof(double));
        if (iv) std::memcpy(iv, r->res.data() + 2 * no, no * sizeof(double));
    } else {
        g_srv_err = r->err;
    }
    if (times) {
        using ms = std::chrono::duration<double, std::milli>;
        // a request that failed before admission has no start time
        const Clock::time_point start = r->t_start.time_since_epoch().count() ? r->t_start : r->t_done;
        times[0] = ms(start - r->t_submit).count();
        times[1] = ms(r->t_done - start).count();
        times[2] = ms(r->t_done - r->t_submit).count();
    }
    s.reqs.erase(it);
    return status;
}

int rbg_server_get_stats(rbg_server* srv, rbg_server_stats* st)
{
    if (!srv || !st) return srv_fail(RBG_ERR_ARG, "null argument");
    Server& s = *srv->s;
    std::lock_guard<std::mutex> lk(s.mu);
    std::memset(st, 0, sizeof(*st));
    st->completed = s.completed;
    st->failed = s.failed;
    st->pending = s.pending.size();
    for (Slot& sl : s.slots) st->in_flight += sl.req ? 1 : 0;
    st->hbm_in_use = s.in_use;
    st->table_cache_hits = s.cache_hits;
    st->table_cache_misses = s.cache_misses;
    st->graph_launches = s.graph_launches;
    st->graph_instantiations = s.graph_instantiations;
    st->graph_updates = s.graph_updates;
    st->max_launch_us = s.max_launch_us;
    st->pin_growths = s.pin_growths;
    st->batches = s.batches;
    st->batched_requests = s.batched_requests;
    st->max_alloc_us = s.max_alloc_us;
    st->max_tables_us = s.max_tables_us;
    st->max_upload_us = s.max_upload_us;
    st->max_graph_us = s.max_graph_us;
    return RBG_OK;
}

int rbg_server_destroy(rbg_server* srv)
{
    if (!srv) return RBG_OK;
    Server& s = *srv->s;
    {
        std::lock_guard<std::mutex> lk(s.mu);
        s.stop = true;
    }
    s.cv_work.notify_all();
    if (s.thr.joinable()) s.thr.join();
    cudaSetDevice(s.dev);
    for (Slot& sl : s.slots) {
        cudaStreamSynchronize(sl.st);
        for (auto& g : sl.graphs) cudaGraphExecDestroy(g.second);
        for (SBuf* b : {&sl.ws, &sl.ivb, &sl.part, &sl.acc, &sl.res, &sl.outs})
            if (b->p) cudaFreeAsync(b->p, sl.st);
        cudaStreamSynchronize(sl.st);
        if (sl.pin) cudaFreeHost(sl.pin);
        cudaEventDestroy(sl.ev);
        cudaStreamDestroy(sl.st);
    }
    for (BatchSlot& b : s.bslots) {
        cudaStreamSynchronize(b.st);
        if (b.graph) cudaGraphExecDestroy(b.graph);
        for (SBuf* x : {&b.in, &b.ivb, &b.part, &b.acc, &b.res})
            if (x->p) cudaFreeAsync(x->p, b.st);
        cudaStreamSynchronize(b.st);
        if (b.pin) cudaFreeHost(b.pin);
        cudaEventDestroy(b.ev);
        cudaStreamDestroy(b.st);
    }
    for (CacheEntry& e : s.cache) {
        if (e.dev) cudaFreeAsync(e.dev, s.copy_st);
        if (e.ready) cudaEventDestroy(e.ready);
    }
    cudaStreamSynchronize(s.copy_st);
    cudaStreamDestroy(s.copy_st);
    if (s.pool) cudaMemPoolDestroy(s.pool);
    delete srv;
    return RBG_OK;
}

}  // extern "C"
