// Continuous-batching training server behind the C ABI (cdlgb_server_*).
//
// The reference trains its datasets one after another: find_motifs_fasta_folder
// (src/CDLmotif.jl:84-93) loops over FASTA files, each through cdl_optimize
// (src/WRAPPER/wrap.jl:1-32).  Here a caller submits datasets at any time from any host
// thread; a request is admitted as soon as a slot is free and its device footprint
// (cdlgb_footprint: the ADMM state and scratch for its N and L) fits in what the
// requests in flight leave of the HBM budget, in arrival order (the oldest waiting
// request is admitted first; a younger one never overtakes it).  Each admitted request
// runs one training -- init, iter_num outer iterations, the code threshold -- on its own
// context and CUDA stream, so the kernels of different datasets overlap on the device;
// its state stays resident until the training ends.  A request whose footprint exceeds
// the whole budget is refused at submission with CDLGB_ENOMEM_BUDGET.  Every kernel is
// deterministic and contexts share no device memory, so a dataset's result does not
// depend on what else is in flight.
#include "cdlgb_internal.h"

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

using clk = std::chrono::steady_clock;

struct Req {
    int64_t id = 0;
    std::vector<float> data;        // (N, 4L) one-hot, copied at submission, or
    std::vector<uint8_t> codes;     // (N, L) one byte per base (FASTA submissions)
    int32_t L4 = 0, N = 0;
    uint64_t footprint = 0;
    int32_t state = CDLGB_REQ_PENDING;
    int32_t status = CDLGB_OK;
    std::string err;
    clk::time_point t_submit, t_admit, t_done;
    // results
    int32_t M = 0, Lg = 0;
    std::vector<float> D_best;      // (Lg, M)
    std::vector<double> objs;       // iter_num
    double obj_best = 0.0, code_thresh = 0.0;
    int32_t outer_done = 0;
    std::vector<float> X_best;      // (Lg, M, N) when the server keeps codes
};

}  // namespace

struct cdlgb_server {
    cdlgb_params p;
    cdlgb_server_config cfg;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::shared_ptr<Req>> pending;
    std::map<int64_t, std::shared_ptr<Req>> reqs;
    uint64_t budget = 0, in_use = 0;
    int running = 0;
    int64_t next_id = 1;
    bool stop = false;
    std::vector<std::thread> workers;
    clk::time_point t0;
    std::mutex emu;                 // guards err (written by failing calls of any thread)
    char err[512];
};

namespace {

// the padded length of the serving form: the smallest L' >= L whose transform length
// 4L' + 8W is one the multi-iteration X-step kernel covers (16 x P and 32 x P for the
// per-lane lengths of xiter_v*.cu) if that costs at most 8 % more transform columns, else the
// smallest whose transform length is a multiple of 16 with prime factors <= 31 (the
// generic in-kernel FFTs)
int friendly_L(int L, int fs) {
    static const int kRegLg[] = {288, 320, 336, 352, 368, 384, 400, 416, 432, 448, 464, 480, 496,
                                 528, 544, 576, 608, 640, 672, 704, 736, 768, 800, 832, 864, 896,
                                 928, 960, 992};
    const int lg = 4 * L + 8 * fs;
    for (int n : kRegLg)
        if (lg <= n && n <= 1.08 * lg && (n - 8 * fs) % 4 == 0) return (n - 8 * fs) / 4;
    auto ok = [](int n) {
        if (n % 16) return false;
        for (int p : {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31})
            while (n % p == 0) n /= p;
        return n == 1;
    };
    int Lp = L;
    while (!ok(4 * Lp + 8 * fs)) ++Lp;
    return Lp;
}

double secs(clk::time_point a, clk::time_point b) {
    return std::chrono::duration<double>(b - a).count();
}

// one training of one dataset on its own context (cdl_optimize's body for one training,
// src/WRAPPER/wrap.jl:5-12)
void train(cdlgb_server* s, Req& r) {
    cdlgb_params p = s->p;
    p.device = s->cfg.device;
    p.hbm_budget_bytes = r.footprint + (1ull << 30);
    cdlgb_ctx* c = nullptr;
    int st = cdlgb_create(&p, &c);
    auto fail = [&](int code) {
        r.status = code;
        r.err = cdlgb_last_error(c);        // this worker's creation message when c is null
    };
    if (st != CDLGB_OK) { fail(st); return; }
    const int iters = s->cfg.iter_num > 0 ? s->cfg.iter_num : p.iter_num;
    int32_t L4 = 0, N = 0, M = 0, gamma = 0, Lg = 0;
    r.objs.assign(iters, 0.0);
    st = r.codes.empty() ? cdlgb_load_data(c, r.data.data(), r.L4, r.N)
                         : load_codes(c, r.codes.data(), r.L4 / 4, r.N);
    if (st != CDLGB_OK ||
        (st = cdlgb_init_state(c, nullptr, nullptr, s->cfg.seed)) != CDLGB_OK ||
        (st = cdlgb_run_outer(c, iters, r.objs.data())) != CDLGB_OK ||
        (st = cdlgb_code_threshold(c, &r.code_thresh)) != CDLGB_OK ||
        (st = cdlgb_dims(c, &L4, &N, &M, &gamma, &Lg)) != CDLGB_OK ||
        (st = cdlgb_get(c, CDLGB_FIELD_OUTER_DONE, &r.outer_done, sizeof(int32_t))) != CDLGB_OK ||
        (st = cdlgb_get(c, CDLGB_FIELD_OBJ_BEST, &r.obj_best, sizeof(double))) != CDLGB_OK) {
        fail(st);
        cdlgb_destroy(c);
        return;
    }
    r.M = M;
    r.Lg = Lg;
    r.objs.resize(r.outer_done);
    r.D_best.resize((size_t)Lg * M);
    st = cdlgb_get(c, CDLGB_FIELD_D_BEST, r.D_best.data(), r.D_best.size() * 4);
    if (st == CDLGB_OK && s->cfg.keep_codes) {
        r.X_best.resize((size_t)Lg * M * N);
        st = cdlgb_get(c, CDLGB_FIELD_X_BEST, r.X_best.data(), r.X_best.size() * 4);
    }
    if (st != CDLGB_OK) fail(st);
    cdlgb_destroy(c);
}

void worker(cdlgb_server* s) {
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        // the oldest pending request, once a slot is free and its footprint fits
        s->cv.wait(lk, [&] {
            return s->stop || (!s->pending.empty() && s->running < s->cfg.slots &&
                               s->in_use + s->pending.front()->footprint <= s->budget);
        });
        if (s->stop) return;        // requests not yet admitted are dropped
        std::shared_ptr<Req> r = s->pending.front();
        s->pending.pop_front();
        s->in_use += r->footprint;
        s->running += 1;
        r->state = CDLGB_REQ_RUNNING;
        r->t_admit = clk::now();
        lk.unlock();
        train(s, *r);
        r->data.clear();
        r->data.shrink_to_fit();
        r->codes.clear();
        r->codes.shrink_to_fit();
        lk.lock();
        r->t_done = clk::now();
        r->state = r->status == CDLGB_OK ? CDLGB_REQ_DONE : CDLGB_REQ_FAILED;
        s->in_use -= r->footprint;
        s->running -= 1;
        s->cv.notify_all();
    }
}

int serr(cdlgb_server* s, int code, const char* msg) {
    if (s) {
        std::lock_guard<std::mutex> lk(s->emu);
        snprintf(s->err, sizeof(s->err), "%s", msg);
    }
    return code;
}

}  // namespace

extern "C" {

int cdlgb_server_create(const cdlgb_params* p, const cdlgb_server_config* cfg, cdlgb_server** out) {
    if (!p || !cfg || !out) return noctx_seterr(CDLGB_EINVAL, "cdlgb_server_create: null argument");
    *out = nullptr;
    if (cfg->slots < 1 || cfg->slots > 64 || cfg->iter_num < 0)
        return noctx_seterr(CDLGB_EINVAL, "cdlgb_server_create: slots=%d (1..64), iter_num=%d (>= 0)",
                            cfg->slots, cfg->iter_num);
    cdlgb_server* s = new (std::nothrow) cdlgb_server();
    if (!s) return noctx_seterr(CDLGB_EINVAL, "cdlgb_server_create: out of host memory");
    s->p = *p;
    s->cfg = *cfg;
    s->err[0] = 0;
    s->budget = cfg->hbm_budget_bytes;
    if (s->budget == 0) {
        size_t fr = 0, tot = 0;
        cudaError_t e = cudaSetDevice(cfg->device);
        if (e == cudaSuccess) e = cudaMemGetInfo(&fr, &tot);
        if (e != cudaSuccess) {
            delete s;
            return noctx_seterr(CDLGB_ECUDA, "cdlgb_server_create: device %d: %s", cfg->device,
                                cudaGetErrorString(e));
        }
        s->budget = (uint64_t)((double)fr * 0.85);
    }
    // the library's device memory pool keeps what finished datasets free for the next
    // ones while the server lives
    devmem_hold(cfg->device, +1);
    s->t0 = clk::now();
    for (int i = 0; i < cfg->slots; ++i) s->workers.emplace_back(worker, s);
    *out = s;
    return CDLGB_OK;
}

namespace {
int enqueue(cdlgb_server* s, std::shared_ptr<Req> r, int64_t* id);
}

int cdlgb_server_submit(cdlgb_server* s, const float* onehot, int32_t L4, int32_t N, int64_t* id) {
    if (!s || !onehot || !id || L4 <= 0 || N <= 0 || L4 % 4)
        return serr(s, CDLGB_EINVAL, "submit: bad arguments");
    auto r = std::make_shared<Req>();
    r->data.assign(onehot, onehot + (size_t)N * L4);
    r->L4 = L4;
    r->N = N;
    return enqueue(s, r, id);
}

int cdlgb_server_submit_fasta(cdlgb_server* s, const char* text, size_t nbytes, int32_t max_entries,
                              int64_t* id) {
    if (!s || !text || !id) return serr(s, CDLGB_EINVAL, "submit_fasta: bad arguments");
    auto r = std::make_shared<Req>();
    int32_t N = 0, L = 0, wrong = 0;
    char err[256];
    int st = fasta_codes(text, nbytes, max_entries, r->codes, &N, &L, &wrong, err, sizeof(err));
    if (st != CDLGB_OK) return serr(s, st, err);
    r->L4 = 4 * L;
    r->N = N;
    return enqueue(s, r, id);
}

namespace {
int enqueue(cdlgb_server* s, std::shared_ptr<Req> r, int64_t* id) {
    if (s->cfg.pad_friendly) {
        // empty columns at the end of every sequence (one-hot zeros, base code 4)
        const int L = r->L4 / 4, Lp = friendly_L(L, s->p.filter_size), N = r->N;
        if (Lp != L) {
            if (!r->codes.empty()) {
                std::vector<uint8_t> c((size_t)N * Lp, 4);
                for (int n = 0; n < N; ++n) memcpy(&c[(size_t)n * Lp], &r->codes[(size_t)n * L], L);
                r->codes.swap(c);
            } else {
                std::vector<float> d((size_t)N * 4 * Lp, 0.f);
                for (int n = 0; n < N; ++n)
                    memcpy(&d[(size_t)n * 4 * Lp], &r->data[(size_t)n * 4 * L], (size_t)4 * L * 4);
                r->data.swap(d);
            }
            r->L4 = 4 * Lp;
        }
    }
    const int32_t L4 = r->L4, N = r->N;
    uint64_t fp = 0;
    int st = cdlgb_footprint(&s->p, L4 / 4, N, &fp);
    if (st != CDLGB_OK) return serr(s, st, "submit: footprint");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return serr(s, CDLGB_ESTATE, "submit: the server is shutting down");
    if (fp > s->budget) {
        char m[200];
        snprintf(m, sizeof(m), "submit: dataset needs %.2f GB, more than the whole budget of %.2f GB",
                 fp / 1e9, s->budget / 1e9);
        return serr(s, CDLGB_ENOMEM_BUDGET, m);
    }
    r->id = s->next_id++;
    r->footprint = fp;
    r->t_submit = clk::now();
    s->reqs[r->id] = r;
    s->pending.push_back(r);
    *id = r->id;
    s->cv.notify_all();
    return CDLGB_OK;
}
}  // namespace

int cdlgb_server_poll(cdlgb_server* s, int64_t id, int32_t wait_ms, cdlgb_request_info* info) {
    if (!s || !info) return CDLGB_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return serr(s, CDLGB_EINVAL, "poll: unknown request id");
    std::shared_ptr<Req> r = it->second;
    if (wait_ms != 0) {
        auto done = [&] { return r->state == CDLGB_REQ_DONE || r->state == CDLGB_REQ_FAILED; };
        if (wait_ms < 0) s->cv.wait(lk, done);
        else s->cv.wait_for(lk, std::chrono::milliseconds(wait_ms), done);
    }
    memset(info, 0, sizeof(*info));
    info->state = r->state;
    info->N = r->N;
    info->L4 = r->L4;
    info->footprint_bytes = r->footprint;
    const auto now = clk::now();
    info->t_submit = secs(s->t0, r->t_submit);
    info->t_admit = r->state == CDLGB_REQ_PENDING ? -1.0 : secs(s->t0, r->t_admit);
    info->t_now = secs(s->t0, now);
    // the results are written by the worker while the request runs, without the lock,
    // and published under it with the final state: read them only then
    if (r->state == CDLGB_REQ_DONE || r->state == CDLGB_REQ_FAILED) {
        info->status = r->status;
        info->M = r->M;
        info->Lg = r->Lg;
        info->outer_done = r->outer_done;
        info->obj_best = r->obj_best;
        info->code_thresh = r->code_thresh;
        info->t_done = secs(s->t0, r->t_done);
        snprintf(info->error, sizeof(info->error), "%s", r->err.c_str());
    } else {
        info->t_done = -1.0;
    }
    return CDLGB_OK;
}

int cdlgb_server_fetch(cdlgb_server* s, int64_t id, float* D_best, size_t D_bytes, double* objs,
                       int32_t objs_cap, float* X_best, size_t X_bytes) {
    if (!s) return CDLGB_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return serr(s, CDLGB_EINVAL, "fetch: unknown request id");
    Req& r = *it->second;
    if (r.state != CDLGB_REQ_DONE) return serr(s, CDLGB_ESTATE, "fetch: request not done");
    if (D_best) {
        if (D_bytes != r.D_best.size() * 4) return serr(s, CDLGB_EINVAL, "fetch: D_best is (Lg, M) float32");
        memcpy(D_best, r.D_best.data(), D_bytes);
    }
    if (objs)
        for (int i = 0; i < objs_cap && i < (int)r.objs.size(); ++i) objs[i] = r.objs[i];
    if (X_best) {
        if (r.X_best.empty()) return serr(s, CDLGB_ESTATE, "fetch: codes not kept (keep_codes = 0)");
        if (X_bytes != r.X_best.size() * 4) return serr(s, CDLGB_EINVAL, "fetch: X_best is (Lg, M, N) float32");
        memcpy(X_best, r.X_best.data(), X_bytes);
    }
    return CDLGB_OK;
}

int cdlgb_server_release(cdlgb_server* s, int64_t id) {
    if (!s) return CDLGB_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return serr(s, CDLGB_EINVAL, "release: unknown request id");
    if (it->second->state != CDLGB_REQ_DONE && it->second->state != CDLGB_REQ_FAILED)
        return serr(s, CDLGB_ESTATE, "release: request still pending or running");
    s->reqs.erase(it);
    return CDLGB_OK;
}

int cdlgb_server_stats(cdlgb_server* s, int32_t* pending, int32_t* running, uint64_t* in_use,
                       uint64_t* budget) {
    if (!s) return CDLGB_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    if (pending) *pending = (int32_t)s->pending.size();
    if (running) *running = s->running;
    if (in_use) *in_use = s->in_use;
    if (budget) *budget = s->budget;
    return CDLGB_OK;
}

// a copy in the calling thread's own buffer: another thread's failing call may rewrite
// the server's message meanwhile
const char* cdlgb_server_last_error(const cdlgb_server* s) {
    static thread_local char buf[512];
    if (!s) {
        const char* m = noctx_err();
        return m ? m : "no server";
    }
    std::lock_guard<std::mutex> lk(const_cast<cdlgb_server*>(s)->emu);
    snprintf(buf, sizeof(buf), "%s", s->err);
    return buf;
}

int cdlgb_server_destroy(cdlgb_server* s) {
    if (!s) return CDLGB_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    for (auto& t : s->workers) t.join();
    devmem_hold(s->cfg.device, -1);
    delete s;
    return CDLGB_OK;
}

}  // extern "C"
