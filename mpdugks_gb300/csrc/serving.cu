// Serving: continuous batching of many DUGKS cases on one GPU.
//
// Three host threads share one server:
//   admission  takes queued cases first in, first out while their device
//              footprint fits the byte budget (and, for batched cases, a slot
//              of the constant-memory case table is free), allocates and
//              initialises each on its own stream, and hands it to a lane;
//   batch lane runs every resident FP32-storage Allen-Cahn case together:
//              each chunk of K steps is one captured CUDA graph, per group
//              of cases with the same model and wall kind, of K persistent
//              launches over a (case slot, tile) table, followed by a launch
//              that advances the cases' step numbers.  Graphs are cached per
//              batch composition.  Cases join and leave at chunk boundaries;
//              a case whose last step falls inside a chunk is skipped by the
//              rest of the chunk's launches;
//   solo lane  runs the other cases (FP64, pseudopotential) one at a time in
//              chunks on a second stream, so their work overlaps the batch.
// A finished case's fields are copied to the host and its device memory is
// freed, which lets the admission thread take the next case.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/dugks_gpu.h"
#include "dugks_device.cuh"
#include "fp32_state.cuh"

namespace dugks {
namespace f32 {
cudaError_t batch_set_case(int slot, const P32 &P, const S32 &S0, cudaStream_t st);
int batch_tiles_of(int nx, int ny);
cudaError_t launch_batch32(int model, int walls, const int2 *tiles, int ntiles, int kstep, const int *case_base,
                           const int *case_stop, cudaStream_t st, int64_t *launches);
cudaError_t launch_batch_advance(int *case_base, const int *slots, int count, int n, cudaStream_t st,
                                 int64_t *launches);
cudaError_t batch_prepare();
}  // namespace f32
namespace internal {
size_t footprint(const dugks_case_t &c, const dugks_grid_t &g);
bool batchable(const dugks_handle_t *h);
void fp32_views(const dugks_handle_t *h, f32::P32 *P, f32::S32 *S);
int64_t steps_done(const dugks_handle_t *h);
int model_of(const dugks_handle_t *h);
int walls_of(const dugks_handle_t *h);
void fp32_adopt_steps(dugks_handle_t *h, int64_t n);
void set_stream(dugks_handle_t *h, cudaStream_t st);
}  // namespace internal
}  // namespace dugks

using namespace dugks;

namespace {

using Clock = std::chrono::steady_clock;

struct SrvCase {
    int64_t id = 0;
    dugks_case_t cs{};
    dugks_grid_t grid{};
    int init_kind = 0;
    std::vector<double> params;
    uint64_t seed = 0;
    int64_t nsteps = 0;
    size_t bytes = 0;
    bool batched = false;
    dugks_handle_t *h = nullptr;
    int slot = -1;
    int64_t base = 0;   // step number at the start of the current chunk (batch lane)
    int64_t base0 = 0;  // step number when the case joined the batch lane
    int state = DUGKS_SRV_QUEUED;
    bool cancel = false;
    double t_submit = 0, t_start = 0, t_done = 0;
    int64_t steps_done = 0;
    std::vector<double> res;  // rho, u, v, phi, p [5][ny][nx]
    std::string err;
};

// one captured chunk: per model group a device tile table, and the graph
struct Chunk {
    std::vector<int> key;  // slot, model, walls, nx, ny of every case (composition)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *dev = nullptr;   // tile tables + slot list
    int64_t launches = 0;  // kernel launches per replay
};

}  // namespace

struct dugks_srv {
    int device = 0;
    size_t max_bytes = 0;
    int chunk = 64;
    Clock::time_point t0;

    std::mutex mu;
    std::condition_variable cv_admit, cv_batch, cv_solo, cv_done;
    bool stopping = false;
    int64_t next_id = 1;
    std::map<int64_t, std::shared_ptr<SrvCase>> cases;
    std::deque<std::shared_ptr<SrvCase>> queue;        // waiting for admission
    std::deque<std::shared_ptr<SrvCase>> ready_batch;  // admitted, waiting for a chunk boundary
    std::deque<std::shared_ptr<SrvCase>> ready_solo;
    size_t bytes_in_use = 0, bytes_peak = 0;
    int slots_used = 0;
    bool slot_busy[f32::BATCH_MAX_CASES] = {};
    int resident = 0, max_resident = 0;
    dugks_srv_stats_t st{};
    std::string err;

    cudaStream_t s_batch = nullptr, s_solo = nullptr, s_prep = nullptr;
    int *d_base = nullptr, *d_stop = nullptr;  // per slot
    int *h_base = nullptr, *h_stop = nullptr;  // pinned staging
    std::vector<Chunk> graphs;                 // cache, most recent last

    std::thread th_admit, th_batch, th_solo;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void set_err(dugks_srv *s, const std::string &m) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->err = m;
}

std::string handle_error(dugks_handle_t *h) {
    char buf[512] = {0};
    dugks_gpu_last_error(h, buf, sizeof(buf));
    return buf;
}

// fields of a finished case to the host, then free its device state
void finish_case(dugks_srv *s, const std::shared_ptr<SrvCase> &c, cudaStream_t st) {
    const size_t n = (size_t)c->grid.nx * c->grid.ny;
    std::vector<double> res(5 * n);
    int rc = DUGKS_OK;
    if (!c->cancel) {
        internal::set_stream(c->h, st);
        rc = dugks_gpu_download(c->h, res.data(), res.data() + n, res.data() + 2 * n, res.data() + 3 * n,
                                res.data() + 4 * n);
    }
    std::string e = rc ? handle_error(c->h) : std::string();
    dugks_gpu_destroy(c->h);
    std::lock_guard<std::mutex> lk(s->mu);
    c->h = nullptr;
    c->t_done = s->now();
    s->bytes_in_use -= c->bytes;
    s->resident -= 1;
    if (c->slot >= 0) {
        s->slot_busy[c->slot] = false;
        s->slots_used -= 1;
        c->slot = -1;
    }
    if (c->cancel) {
        c->state = DUGKS_SRV_CANCELLED;
        s->st.cancelled += 1;
    } else if (rc) {
        c->state = DUGKS_SRV_FAILED;
        c->err = e;
        s->st.failed += 1;
    } else {
        c->res = std::move(res);
        c->steps_done = c->nsteps;
        c->state = DUGKS_SRV_DONE;
        s->st.completed += 1;
        s->st.cell_updates += c->nsteps * (int64_t)n;
    }
    s->cv_admit.notify_all();
    s->cv_done.notify_all();
}

void fail_case(dugks_srv *s, const std::shared_ptr<SrvCase> &c, const std::string &why, bool admitted) {
    if (c->h) dugks_gpu_destroy(c->h);
    std::lock_guard<std::mutex> lk(s->mu);
    c->h = nullptr;
    c->state = DUGKS_SRV_FAILED;
    c->err = why;
    c->t_done = s->now();
    s->st.failed += 1;
    if (admitted) {
        s->bytes_in_use -= c->bytes;
        s->resident -= 1;
        if (c->slot >= 0) {
            s->slot_busy[c->slot] = false;
            s->slots_used -= 1;
            c->slot = -1;
        }
    }
    s->cv_admit.notify_all();
    s->cv_done.notify_all();
}

// ---- admission: FIFO by footprint
void admit_loop(dugks_srv *s) {
    cudaSetDevice(s->device);
    for (;;) {
        std::shared_ptr<SrvCase> c;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_admit.wait(lk, [&] {
                if (s->stopping) return true;
                if (s->queue.empty()) return false;
                const auto &h = s->queue.front();
                if (h->cancel) return true;
                const bool fits = s->bytes_in_use + h->bytes <= s->max_bytes;
                const bool slot = !h->batched || s->slots_used < f32::BATCH_MAX_CASES;
                return fits && slot;
            });
            if (s->stopping) return;
            c = s->queue.front();
            s->queue.pop_front();
            if (c->cancel) {
                c->state = DUGKS_SRV_CANCELLED;
                c->t_done = s->now();
                s->st.cancelled += 1;
                s->cv_done.notify_all();
                continue;
            }
            s->bytes_in_use += c->bytes;
            s->bytes_peak = std::max(s->bytes_peak, s->bytes_in_use);
            s->resident += 1;
            s->max_resident = std::max(s->max_resident, s->resident);
            if (c->batched) {
                for (int k = 0; k < f32::BATCH_MAX_CASES; ++k)
                    if (!s->slot_busy[k]) {
                        s->slot_busy[k] = true;
                        c->slot = k;
                        break;
                    }
                s->slots_used += 1;
            }
            c->state = DUGKS_SRV_RUNNING;
            c->t_start = s->now();
        }
        dugks_handle_t *h = nullptr;
        int rc = dugks_gpu_create(&c->cs, &c->grid, &h);
        if (rc) {
            char buf[512] = {0};
            dugks_gpu_last_error(nullptr, buf, sizeof(buf));
            fail_case(s, c, buf, true);
            continue;
        }
        c->h = h;
        internal::set_stream(h, s->s_prep);
        rc = dugks_gpu_init(h, c->init_kind, c->params.empty() ? nullptr : c->params.data(), (int)c->params.size(),
                            c->seed);
        if (rc) {
            fail_case(s, c, handle_error(h), true);
            continue;
        }
        std::lock_guard<std::mutex> lk(s->mu);
        if (c->batched) {
            s->ready_batch.push_back(c);
            s->cv_batch.notify_all();
        } else {
            s->ready_solo.push_back(c);
            s->cv_solo.notify_all();
        }
    }
}

// ---- batch lane
cudaError_t capture_chunk(dugks_srv *s, const std::vector<std::shared_ptr<SrvCase>> &act, Chunk &ch) {
    // group the cases by (model, walls); tile table per group, slot list at the end
    std::map<std::pair<int, int>, std::vector<int2>> groups;
    std::vector<int> slots;
    for (const auto &c : act) {
        const int m = internal::model_of(c->h), w = internal::walls_of(c->h);
        auto &tb = groups[{m, w}];
        const int nt = f32::batch_tiles_of(c->grid.nx, c->grid.ny);
        for (int t = 0; t < nt; ++t) tb.push_back(make_int2(c->slot, t));
        slots.push_back(c->slot);
    }
    size_t total = 0;
    for (auto &g : groups) total += g.second.size() * sizeof(int2);
    const size_t slot_off = (total + 255) & ~(size_t)255;
    total = slot_off + slots.size() * sizeof(int);
    cudaError_t e = cudaMalloc(&ch.dev, total);
    if (e != cudaSuccess) return e;
    std::vector<char> host(total);
    size_t off = 0;
    std::vector<std::pair<std::pair<int, int>, std::pair<size_t, int>>> where;  // group -> (offset, count)
    for (auto &g : groups) {
        std::memcpy(host.data() + off, g.second.data(), g.second.size() * sizeof(int2));
        where.push_back({g.first, {off, (int)g.second.size()}});
        off += g.second.size() * sizeof(int2);
    }
    std::memcpy(host.data() + slot_off, slots.data(), slots.size() * sizeof(int));
    if ((e = cudaMemcpy(ch.dev, host.data(), total, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
    char *base = static_cast<char *>(ch.dev);
    int64_t launches = 0;
    if ((e = cudaStreamBeginCapture(s->s_batch, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    cudaError_t le = cudaSuccess;
    for (int k = 0; k < s->chunk && le == cudaSuccess; ++k)
        for (auto &g : where) {
            le = f32::launch_batch32(g.first.first, g.first.second, reinterpret_cast<const int2 *>(base + g.second.first),
                                     g.second.second, k, s->d_base, s->d_stop, s->s_batch, &launches);
            if (le != cudaSuccess) break;
        }
    if (le == cudaSuccess)
        le = f32::launch_batch_advance(s->d_base, reinterpret_cast<const int *>(base + slot_off), (int)slots.size(),
                                       s->chunk, s->s_batch, &launches);
    e = cudaStreamEndCapture(s->s_batch, &ch.graph);
    if (le != cudaSuccess) return le;
    if (e != cudaSuccess) return e;
    if ((e = cudaGraphInstantiate(&ch.exec, ch.graph, 0)) != cudaSuccess) return e;
    ch.launches = launches;
    std::lock_guard<std::mutex> lk(s->mu);
    s->st.graphs_captured += 1;
    return cudaSuccess;
}

void free_chunk(Chunk &ch) {
    if (ch.exec) cudaGraphExecDestroy(ch.exec);
    if (ch.graph) cudaGraphDestroy(ch.graph);
    if (ch.dev) cudaFree(ch.dev);
    ch = Chunk{};
}

void batch_loop(dugks_srv *s) {
    cudaSetDevice(s->device);
    std::vector<std::shared_ptr<SrvCase>> act;
    for (;;) {
        // take the cases that became ready; drop cancelled ones
        std::vector<std::shared_ptr<SrvCase>> joined, leaving;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_batch.wait(lk, [&] { return s->stopping || !act.empty() || !s->ready_batch.empty(); });
            if (s->stopping && s->ready_batch.empty() && act.empty()) return;
            while (!s->ready_batch.empty()) {
                joined.push_back(s->ready_batch.front());
                s->ready_batch.pop_front();
            }
            for (auto &c : act)
                if (c->cancel || s->stopping) leaving.push_back(c);
            for (auto &c : joined)
                if (c->cancel || s->stopping) leaving.push_back(c);
        }
        for (auto &c : joined) {
            if (c->cancel || s->stopping) continue;
            f32::P32 P;
            f32::S32 S;
            internal::fp32_views(c->h, &P, &S);
            c->base = c->base0 = internal::steps_done(c->h);
            s->h_base[c->slot] = (int)c->base;
            s->h_stop[c->slot] = (int)c->nsteps;
            cudaError_t e = f32::batch_set_case(c->slot, P, S, s->s_batch);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(s->d_base + c->slot, s->h_base + c->slot, sizeof(int), cudaMemcpyHostToDevice,
                                    s->s_batch);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(s->d_stop + c->slot, s->h_stop + c->slot, sizeof(int), cudaMemcpyHostToDevice,
                                    s->s_batch);
            if (e != cudaSuccess) {
                fail_case(s, c, std::string("batch admission: ") + cudaGetErrorString(e), true);
                continue;
            }
            act.push_back(c);
        }
        for (auto &c : leaving) {
            auto it = std::find(act.begin(), act.end(), c);
            if (it != act.end()) act.erase(it);
            if (c->h) finish_case(s, c, s->s_batch);
        }
        if (act.empty()) continue;
        // the composition's graph (cached)
        std::vector<int> key;
        for (auto &c : act) {
            key.push_back(c->slot);
            key.push_back(internal::model_of(c->h));
            key.push_back(internal::walls_of(c->h));
            key.push_back(c->grid.nx);
            key.push_back(c->grid.ny);
        }
        int gi = -1;
        for (size_t k = 0; k < s->graphs.size(); ++k)
            if (s->graphs[k].key == key) gi = (int)k;
        if (gi < 0) {
            if (s->graphs.size() >= 8) {
                cudaStreamSynchronize(s->s_batch);
                free_chunk(s->graphs.front());
                s->graphs.erase(s->graphs.begin());
            }
            Chunk ch;
            ch.key = key;
            cudaError_t e = capture_chunk(s, act, ch);
            if (e != cudaSuccess) {
                free_chunk(ch);
                const std::string why = std::string("chunk capture: ") + cudaGetErrorString(e);
                set_err(s, why);
                for (auto &c : act) fail_case(s, c, why, true);
                act.clear();
                continue;
            }
            s->graphs.push_back(ch);
            gi = (int)s->graphs.size() - 1;
        }
        const auto t_chunk = Clock::now();
        cudaError_t e = cudaGraphLaunch(s->graphs[gi].exec, s->s_batch);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->s_batch);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->st.chunks += 1;
            s->st.launches += s->graphs[gi].launches;
            s->st.busy_s += std::chrono::duration<double>(Clock::now() - t_chunk).count();
        }
        if (e != cudaSuccess) {
            const std::string why = std::string("chunk launch: ") + cudaGetErrorString(e);
            set_err(s, why);
            for (auto &c : act) fail_case(s, c, why, true);
            act.clear();
            continue;
        }
        // advance the host copies of the step numbers; finished cases leave
        std::vector<std::shared_ptr<SrvCase>> done;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (auto &c : act) {
                c->base += s->chunk;
                c->steps_done = std::min(c->base, c->nsteps);
                if (c->base >= c->nsteps) {
                    // the launches past the case's last step skipped it
                    internal::fp32_adopt_steps(c->h, std::max<int64_t>(c->nsteps - c->base0, 0));
                    done.push_back(c);
                }
            }
        }
        for (auto &c : done) {
            act.erase(std::find(act.begin(), act.end(), c));
            finish_case(s, c, s->s_batch);
        }
    }
}

// ---- solo lane
void solo_loop(dugks_srv *s) {
    cudaSetDevice(s->device);
    for (;;) {
        std::shared_ptr<SrvCase> c;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_solo.wait(lk, [&] { return s->stopping || !s->ready_solo.empty(); });
            if (s->ready_solo.empty()) return;
            c = s->ready_solo.front();
            s->ready_solo.pop_front();
        }
        int rc = DUGKS_OK;
        while (rc == DUGKS_OK && !c->cancel && !s->stopping && c->steps_done < c->nsteps) {
            const int n = (int)std::min<int64_t>(s->chunk, c->nsteps - c->steps_done);
            rc = dugks_gpu_step(c->h, n, s->s_solo);
            if (rc == DUGKS_OK && cudaStreamSynchronize(s->s_solo) != cudaSuccess) rc = DUGKS_ECUDA;
            std::lock_guard<std::mutex> lk(s->mu);
            c->steps_done += n;
        }
        if (s->stopping) c->cancel = true;
        if (rc) fail_case(s, c, handle_error(c->h), true);
        else finish_case(s, c, s->s_solo);
    }
}

std::shared_ptr<SrvCase> find(dugks_srv *s, int64_t id) {
    auto it = s->cases.find(id);
    return it == s->cases.end() ? nullptr : it->second;
}

void fill_status(const SrvCase &c, dugks_srv_status_t *st) {
    st->state = c.state;
    st->batched = c.batched ? 1 : 0;
    st->nsteps = c.nsteps;
    st->steps_done = c.steps_done;
    st->bytes = c.bytes;
    st->t_submit = c.t_submit;
    st->t_start = c.t_start;
    st->t_done = c.t_done;
}

bool terminal(int state) { return state >= DUGKS_SRV_DONE; }

}  // namespace

extern "C" int dugks_srv_create(const dugks_srv_config_t *cfg, dugks_srv_t **out) {
    if (!out) return DUGKS_EINVAL;
    *out = nullptr;
    auto *s = new (std::nothrow) dugks_srv();
    if (!s) return DUGKS_ENOMEM;
    s->t0 = Clock::now();
    cudaError_t e = cudaGetDevice(&s->device);
    size_t freeb = 0, totb = 0;
    if (e == cudaSuccess) e = cudaMemGetInfo(&freeb, &totb);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_batch, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_solo, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_prep, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = f32::batch_prepare();  // kernel attributes, before any stream capture
    if (e == cudaSuccess) e = cudaMalloc(&s->d_base, 2 * f32::BATCH_MAX_CASES * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_base, 2 * f32::BATCH_MAX_CASES * sizeof(int));
    if (e != cudaSuccess) {
        dugks_srv_destroy(s);
        return DUGKS_ECUDA;
    }
    s->d_stop = s->d_base + f32::BATCH_MAX_CASES;
    s->h_stop = s->h_base + f32::BATCH_MAX_CASES;
    std::memset(s->h_base, 0, 2 * f32::BATCH_MAX_CASES * sizeof(int));
    cudaMemset(s->d_base, 0, 2 * f32::BATCH_MAX_CASES * sizeof(int));
    s->max_bytes = (cfg && cfg->max_bytes) ? cfg->max_bytes : (size_t)(0.85 * (double)freeb);
    s->chunk = (cfg && cfg->chunk_steps > 0) ? cfg->chunk_steps : 64;
    s->th_admit = std::thread(admit_loop, s);
    s->th_batch = std::thread(batch_loop, s);
    s->th_solo = std::thread(solo_loop, s);
    *out = s;
    return DUGKS_OK;
}

extern "C" int dugks_srv_submit(dugks_srv_t *s, const dugks_case_t *c, const dugks_grid_t *g, int init_kind,
                                const double *params, int nparams, uint64_t seed, int64_t nsteps, int64_t *id) {
    if (!s || !c || !g || !id || nsteps < 0 || nparams < 0 || (nparams > 0 && !params)) return DUGKS_EINVAL;
    if (g->nx < 3 || g->ny < 3) return DUGKS_EINVAL;
    if (nsteps > (int64_t)0x7fffffff - 4 * 1024) return DUGKS_EINVAL;  // step numbers are 32-bit on the device
    auto k = std::make_shared<SrvCase>();
    k->cs = *c;
    k->grid = *g;
    k->init_kind = init_kind;
    k->params.assign(params, params + nparams);
    k->seed = seed;
    k->nsteps = nsteps;
    k->bytes = internal::footprint(*c, *g);
    k->batched = c->precision == DUGKS_FP32_DEV && (c->model == DUGKS_MODEL_AC || c->model == DUGKS_MODEL_HCZ);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return DUGKS_EINVAL;
    if (k->bytes > s->max_bytes) {
        s->err = "case footprint " + std::to_string(k->bytes) + " B exceeds the server budget " +
                 std::to_string(s->max_bytes) + " B";
        return DUGKS_ENOMEM;
    }
    k->id = s->next_id++;
    k->t_submit = s->now();
    s->cases[k->id] = k;
    s->queue.push_back(k);
    s->st.submitted += 1;
    s->cv_admit.notify_all();
    *id = k->id;
    return DUGKS_OK;
}

extern "C" int dugks_srv_poll(dugks_srv_t *s, int64_t id, dugks_srv_status_t *st) {
    if (!s || !st) return DUGKS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto c = find(s, id);
    if (!c) return DUGKS_EINVAL;
    fill_status(*c, st);
    return DUGKS_OK;
}

extern "C" int dugks_srv_wait(dugks_srv_t *s, int64_t id, double timeout_s, dugks_srv_status_t *st) {
    if (!s) return DUGKS_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto c = find(s, id);
    if (!c) return DUGKS_EINVAL;
    auto ok = [&] { return terminal(c->state); };
    if (timeout_s < 0) {
        s->cv_done.wait(lk, ok);
    } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ok)) {
        if (st) fill_status(*c, st);
        return DUGKS_ETIMEOUT;
    }
    if (st) fill_status(*c, st);
    return DUGKS_OK;
}

extern "C" int dugks_srv_result(dugks_srv_t *s, int64_t id, double *rho, double *u, double *v, double *phi,
                                double *p) {
    if (!s) return DUGKS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto c = find(s, id);
    if (!c || c->state != DUGKS_SRV_DONE) return DUGKS_EINVAL;
    const size_t n = (size_t)c->grid.nx * c->grid.ny;
    double *dst[5] = {rho, u, v, phi, p};
    for (int k = 0; k < 5; ++k)
        if (dst[k]) std::memcpy(dst[k], c->res.data() + k * n, n * sizeof(double));
    return DUGKS_OK;
}

extern "C" int dugks_srv_release(dugks_srv_t *s, int64_t id) {
    if (!s) return DUGKS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto c = find(s, id);
    if (!c || !terminal(c->state)) return DUGKS_EINVAL;
    s->cases.erase(id);
    return DUGKS_OK;
}

extern "C" int dugks_srv_cancel(dugks_srv_t *s, int64_t id) {
    if (!s) return DUGKS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    auto c = find(s, id);
    if (!c) return DUGKS_EINVAL;
    if (terminal(c->state)) return DUGKS_OK;
    c->cancel = true;
    s->cv_admit.notify_all();
    s->cv_batch.notify_all();
    return DUGKS_OK;
}

extern "C" int dugks_srv_stats(dugks_srv_t *s, dugks_srv_stats_t *out) {
    if (!s || !out) return DUGKS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->max_resident = s->max_resident;
    out->bytes_in_use = s->bytes_in_use;
    out->bytes_peak = s->bytes_peak;
    out->max_bytes = s->max_bytes;
    return DUGKS_OK;
}

extern "C" int dugks_srv_last_error(dugks_srv_t *s, char *buf, size_t len) {
    if (!s || !buf || !len) return DUGKS_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    std::strncpy(buf, s->err.c_str(), len - 1);
    buf[len - 1] = 0;
    return DUGKS_OK;
}

extern "C" int dugks_srv_destroy(dugks_srv_t *s) {
    if (!s) return DUGKS_EINVAL;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        for (auto &kv : s->cases)
            if (!terminal(kv.second->state)) kv.second->cancel = true;
        s->cv_admit.notify_all();
        s->cv_batch.notify_all();
        s->cv_solo.notify_all();
    }
    if (s->th_admit.joinable()) s->th_admit.join();
    if (s->th_batch.joinable()) s->th_batch.join();
    if (s->th_solo.joinable()) s->th_solo.join();
    // cases admitted but never picked up by a lane
    for (auto *dq : {&s->ready_batch, &s->ready_solo})
        for (auto &c : *dq)
            if (c->h) {
                dugks_gpu_destroy(c->h);
                c->h = nullptr;
            }
    for (auto &ch : s->graphs) free_chunk(ch);
    if (s->s_batch) cudaStreamSynchronize(s->s_batch);
    if (s->d_base) cudaFree(s->d_base);
    if (s->h_base) cudaFreeHost(s->h_base);
    for (cudaStream_t st : {s->s_batch, s->s_solo, s->s_prep})
        if (st) cudaStreamDestroy(st);
    delete s;
    return DUGKS_OK;
}
