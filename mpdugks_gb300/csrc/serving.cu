// Serving: continuous batching of many DUGKS cases on one GPU.
//
// Host threads of one server:
//   admission   takes queued cases first in, first out while their device
//               footprint fits the byte budget (and, for batched cases, a slot
//               of the constant-memory case table is free), allocates and
//               initialises each on its own stream, and hands it to a lane;
//   batch lane  runs every resident FP32-storage Allen-Cahn case together:
//               each chunk of K steps is one captured CUDA graph, per group
//               of cases with the same model and wall kind, of K persistent
//               launches over a (case slot, tile) table, followed by a launch
//               that advances the cases' step numbers.  Graphs are cached per
//               batch composition.  Cases join and leave at chunk boundaries;
//               a case whose next stop (a check, a snapshot, its last step)
//               falls inside a chunk is skipped by the rest of the chunk's
//               launches;
//   solo lanes  run the other cases (FP64, pseudopotential), one case per lane
//               at a time, each lane on its own stream, so their work overlaps
//               one another and the batch;
//   writer      formats and writes FlowField files from pinned host copies of
//               the fields while the cases run on.
// Every `check_every` steps a case's density residual and finiteness are
// checked, like the reference's residual control (Ark/Cpp/DUGKS2DSolver.cpp:164,
// Update_Residual :807-835): it stops converged at or below its tolerance and
// fails when its state is no longer finite.  A finished case's fields are
// copied to the host and its device memory is freed, which lets the admission
// thread take the next case.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/dugks_gpu.h"
#include "../host/flowfield.hpp"
#include "dugks_device.cuh"
#include "fp32_state.cuh"
#include "trace.hpp"

namespace dugks {
namespace f32 {
cudaError_t batch_set_case(int slot, const P32 &P, const S32 &S, int64_t step, cudaStream_t st);
int batch_tiles_of(int nx, int ny);
cudaError_t launch_batch32(int model, int walls, const int2 *tiles, int ntiles, int kstep, const int *case_base,
                           const int *case_stop, cudaStream_t st, int64_t *launches);
cudaError_t launch_streamb32(int model, int walls, const int4 *items, int nitems, int kstep, const int *case_base,
                             const int *case_stop, cudaStream_t st, int64_t *launches);
void stream_batch_items(const std::vector<int3> &cases, std::vector<int4> &items);
cudaError_t launch_batch_advance(int *case_base, const int *slots, int count, int n, cudaStream_t st,
                                 int64_t *launches);
cudaError_t batch_prepare();
}  // namespace f32
namespace internal {
size_t footprint(const dugks_case_t &c, const dugks_grid_t &g);
void fp32_views(const dugks_handle_t *h, f32::P32 *P, f32::S32 *S);
int64_t steps_done(const dugks_handle_t *h);
int model_of(const dugks_handle_t *h);
int walls_of(const dugks_handle_t *h);
double dt_of(const dugks_handle_t *h);
void fp32_adopt_steps(dugks_handle_t *h, int64_t n);
void set_stream(dugks_handle_t *h, cudaStream_t st);
}  // namespace internal
}  // namespace dugks

using namespace dugks;

namespace {

using Clock = std::chrono::steady_clock;

constexpr int DEFAULT_CHECK_EVERY = 1000;  // ResidualControl, Ark/Constant/ZeroNamespace.h:175
constexpr int FLOWFIELD_FIELDS = 8;        // rho, u, v, phi, p, tau, Fx, Fy
constexpr size_t WRITER_MAX_PENDING = (size_t)1 << 30;  // bytes of fields waiting for the writer

struct Pinned {
    double *p = nullptr;
    size_t n = 0;  // doubles
};

struct SrvCase {
    int64_t id = 0;
    dugks_case_t cs{};
    dugks_grid_t grid{};
    int init_kind = 0;
    std::vector<double> params;
    uint64_t seed = 0;
    int64_t nsteps = 0;
    double residual_tol = 0;
    int check_every = DEFAULT_CHECK_EVERY;
    int snapshot_every = 0;
    std::string out_dir;  // empty: no files
    double dt = 0.5;
    size_t bytes = 0;
    bool batched = false;
    dugks_handle_t *h = nullptr;
    int slot = -1;
    int64_t base = 0;   // batch lane: step number at the start of the current chunk
    int64_t dstop = 0;  // batch lane: the step at which the case next stops (check, snapshot, last step)
    int state = DUGKS_SRV_QUEUED;
    bool cancel = false;
    int stop_reason = DUGKS_SRV_STOP_NONE;
    int files = 0;
    double residual = -1.0;
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

// fields of one case at one step, waiting for the writer
struct WriteJob {
    std::shared_ptr<SrvCase> c;
    int64_t step = 0;
    Pinned buf;
    bool final = false;  // the case's last file: the case ends when it is written
};

}  // namespace

struct dugks_srv {
    int device = 0;
    size_t max_bytes = 0;
    int chunk = 50;
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

    cudaStream_t s_batch = nullptr, s_prep = nullptr;
    std::vector<cudaStream_t> s_solo;
    int *d_base = nullptr, *d_stop = nullptr;  // per slot
    int *h_base = nullptr, *h_stop = nullptr;  // pinned staging
    std::vector<Chunk> graphs;                 // cache, most recent last

    // writer: jobs, pinned buffers and their pool (own lock; never held with mu)
    std::mutex wmu;
    std::condition_variable cv_job, cv_space;
    std::deque<WriteJob> jobs;
    std::vector<Pinned> pool, pinned_all;
    size_t pending_bytes = 0;
    bool writer_stop = false;

    std::thread th_admit, th_batch, th_writer;
    std::vector<std::thread> th_solo;

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

// ---- pinned host buffers for field copies (reused; freed with the server)
Pinned take_pinned(dugks_srv *s, size_t n) {
    std::unique_lock<std::mutex> lk(s->wmu);
    // back-pressure: wait while the writer holds too many bytes
    s->cv_space.wait(lk, [&] { return s->pending_bytes == 0 || s->pending_bytes + n * 8 <= WRITER_MAX_PENDING; });
    int best = -1;
    for (int k = 0; k < (int)s->pool.size(); ++k)
        if (s->pool[k].n >= n && (best < 0 || s->pool[k].n < s->pool[best].n)) best = k;
    if (best >= 0) {
        Pinned b = s->pool[best];
        s->pool.erase(s->pool.begin() + best);
        return b;
    }
    Pinned b;
    if (cudaMallocHost(reinterpret_cast<void **>(&b.p), n * sizeof(double)) != cudaSuccess) return Pinned{};
    b.n = n;
    s->pinned_all.push_back(b);
    return b;
}

void give_pinned(dugks_srv *s, Pinned b) {
    if (!b.p) return;
    std::lock_guard<std::mutex> lk(s->wmu);
    s->pool.push_back(b);
}

// the FlowField fields of a case into `b` ([8][ny][nx]: rho, u, v, phi, p, tau, Fx, Fy;
// the first five only when nf == 5)
int gather(const std::shared_ptr<SrvCase> &c, cudaStream_t st, double *b, int nf) {
    const size_t n = (size_t)c->grid.nx * c->grid.ny;
    internal::set_stream(c->h, st);
    int rc = dugks_gpu_download(c->h, b, b + n, b + 2 * n, b + 3 * n, b + 4 * n);
    if (rc == DUGKS_OK && nf > 5) rc = dugks_gpu_get_field(c->h, DUGKS_F_TAU, b + 5 * n);
    if (rc == DUGKS_OK && nf > 5) rc = dugks_gpu_get_field(c->h, DUGKS_F_FX, b + 6 * n);
    if (rc == DUGKS_OK && nf > 5) rc = dugks_gpu_get_field(c->h, DUGKS_F_FY, b + 7 * n);
    return rc;
}

void enqueue_write(dugks_srv *s, WriteJob j) {
    std::lock_guard<std::mutex> lk(s->wmu);
    s->pending_bytes += j.buf.n * sizeof(double);
    s->jobs.push_back(std::move(j));
    s->cv_job.notify_all();
}

// a FlowField file of the case's current state (step `step`), written by the writer thread
int snapshot(dugks_srv *s, const std::shared_ptr<SrvCase> &c, cudaStream_t st, int64_t step) {
    const size_t n = (size_t)c->grid.nx * c->grid.ny;
    Pinned b = take_pinned(s, FLOWFIELD_FIELDS * n);
    if (!b.p) return DUGKS_ENOMEM;
    const int rc = gather(c, st, b.p, FLOWFIELD_FIELDS);
    if (rc) {
        give_pinned(s, b);
        return rc;
    }
    enqueue_write(s, WriteJob{c, step, b, false});
    return DUGKS_OK;
}

void mark_done(dugks_srv *s, const std::shared_ptr<SrvCase> &c) {
    // with s->mu held
    c->state = DUGKS_SRV_DONE;
    c->t_done = s->now();
    s->st.completed += 1;
    if (c->stop_reason == DUGKS_SRV_STOP_CONVERGED) s->st.converged += 1;
    s->cv_done.notify_all();
}

void writer_loop(dugks_srv *s) {
    for (;;) {
        WriteJob j;
        {
            std::unique_lock<std::mutex> lk(s->wmu);
            s->cv_job.wait(lk, [&] { return s->writer_stop || !s->jobs.empty(); });
            if (s->jobs.empty()) return;
            j = std::move(s->jobs.front());
            s->jobs.pop_front();
        }
        const auto &c = j.c;
        const size_t n = (size_t)c->grid.nx * c->grid.ny;
        std::string why;
        try {
            TraceRange trace("srv FlowField write");
            dugks_host::FlowField ff;
            ff.cells = n;
            const double *b = j.buf.p;
            ff.rho.assign(b, b + n);
            ff.u.assign(b + n, b + 2 * n);
            ff.v.assign(b + 2 * n, b + 3 * n);
            ff.phi.assign(b + 3 * n, b + 4 * n);
            ff.p.assign(b + 4 * n, b + 5 * n);
            ff.tau.assign(b + 5 * n, b + 6 * n);
            ff.fx.assign(b + 6 * n, b + 7 * n);
            ff.fy.assign(b + 7 * n, b + 8 * n);
            ff.T.assign(n, 1.0 / 3.0);  // isothermal models keep the reference temperature T0
            const std::string name = dugks_host::flowfield_name(j.step, (double)j.step * c->dt, "0", "Car",
                                                                std::to_string(c->grid.nx), "0.5");
            dugks_host::write_flowfield(c->out_dir + "/" + name, ff);
        } catch (const std::exception &e) {
            why = std::string("FlowField output: ") + e.what();
        }
        {
            std::lock_guard<std::mutex> lk(s->wmu);
            s->pending_bytes -= j.buf.n * sizeof(double);
            s->pool.push_back(j.buf);
            s->cv_space.notify_all();
        }
        std::lock_guard<std::mutex> lk(s->mu);
        if (why.empty()) {
            c->files += 1;
            s->st.files_written += 1;
        } else if (c->err.empty()) {
            c->err = why;
            s->err = why;
        }
        if (j.final) {
            if (c->err.empty()) {
                mark_done(s, c);
            } else {
                c->state = DUGKS_SRV_FAILED;
                c->t_done = s->now();
                s->st.failed += 1;
                s->cv_done.notify_all();
            }
        }
    }
}

// the next step at which the case stops on its lane: a check, a snapshot or its last step
int64_t next_stop(const SrvCase &c, int64_t step) {
    int64_t t = c.nsteps;
    if (c.check_every > 0) t = std::min(t, (step / c.check_every + 1) * c.check_every);
    if (!c.out_dir.empty() && c.snapshot_every > 0) t = std::min(t, (step / c.snapshot_every + 1) * c.snapshot_every);
    return std::max(t, step);
}

// the case reached a stop (c->steps_done): check, snapshot; true when it ends here
bool at_stop(dugks_srv *s, const std::shared_ptr<SrvCase> &c, cudaStream_t st, int *rc) {
    const int64_t step = c->steps_done;
    bool end = step >= c->nsteps;
    if (c->check_every > 0 && step > 0 && step % c->check_every == 0) {
        internal::set_stream(c->h, st);
        dugks_reductions_t r{};
        *rc = dugks_gpu_reduce(c->h, &r);
        if (*rc) return true;
        std::lock_guard<std::mutex> lk(s->mu);
        c->residual = r.residual;
        if (!std::isfinite(r.sum_rho) || !std::isfinite(r.residual)) {
            c->stop_reason = DUGKS_SRV_STOP_DIVERGED;
            return true;
        }
        if (c->residual_tol > 0 && r.residual <= c->residual_tol) {
            c->stop_reason = DUGKS_SRV_STOP_CONVERGED;
            end = true;
        }
    }
    if (!end && !c->out_dir.empty() && c->snapshot_every > 0 && step % c->snapshot_every == 0) {
        *rc = snapshot(s, c, st, step);
        if (*rc) return true;
    }
    return end;
}

// release a case's device memory and slot (with s->mu held)
void release_device(dugks_srv *s, const std::shared_ptr<SrvCase> &c) {
    c->h = nullptr;
    s->bytes_in_use -= c->bytes;
    s->resident -= 1;
    if (c->slot >= 0) {
        s->slot_busy[c->slot] = false;
        s->slots_used -= 1;
        c->slot = -1;
    }
    s->cv_admit.notify_all();
}

// a case leaves its lane: fields to the host (and to the writer), device state freed
void finish_case(dugks_srv *s, const std::shared_ptr<SrvCase> &c, cudaStream_t st, int rc) {
    const size_t n = (size_t)c->grid.nx * c->grid.ny;
    const bool diverged = c->stop_reason == DUGKS_SRV_STOP_DIVERGED;
    const bool files = !c->out_dir.empty();
    std::string e = rc ? handle_error(c->h) : std::string();
    Pinned b;
    if (!c->cancel && !rc && !diverged) {
        b = take_pinned(s, (files ? FLOWFIELD_FIELDS : 5) * n);
        if (!b.p) {
            rc = DUGKS_ENOMEM;
            e = "no pinned host memory for the result";
        } else if ((rc = gather(c, st, b.p, files ? FLOWFIELD_FIELDS : 5)) != DUGKS_OK) {
            e = handle_error(c->h);
        }
    }
    dugks_gpu_destroy(c->h);
    std::vector<double> res;
    if (!c->cancel && !rc && !diverged) res.assign(b.p, b.p + 5 * n);
    std::unique_lock<std::mutex> lk(s->mu);
    release_device(s, c);
    const bool counted = !c->cancel && !rc;
    if (counted) s->st.cell_updates += c->steps_done * (int64_t)n;
    if (c->cancel) {
        c->state = DUGKS_SRV_CANCELLED;
        s->st.cancelled += 1;
    } else if (rc || diverged) {
        c->state = DUGKS_SRV_FAILED;
        c->err = rc ? e : "non-finite state at step " + std::to_string(c->steps_done);
        s->st.failed += 1;
        if (diverged) s->st.diverged += 1;
    } else {
        c->res = std::move(res);
        if (files) {  // ends when the writer has written its last file
            lk.unlock();
            enqueue_write(s, WriteJob{c, c->steps_done, b, true});
            return;
        }
        mark_done(s, c);
    }
    if (c->state != DUGKS_SRV_DONE) c->t_done = s->now();
    s->cv_done.notify_all();
    lk.unlock();
    give_pinned(s, b);
}

void fail_case(dugks_srv *s, const std::shared_ptr<SrvCase> &c, const std::string &why, bool admitted) {
    if (c->h) dugks_gpu_destroy(c->h);
    std::lock_guard<std::mutex> lk(s->mu);
    c->h = nullptr;
    c->state = DUGKS_SRV_FAILED;
    c->err = why;
    c->t_done = s->now();
    s->st.failed += 1;
    if (admitted) release_device(s, c);
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
        c->dt = internal::dt_of(h);
        internal::set_stream(h, s->s_prep);
        rc = dugks_gpu_init(h, c->init_kind, c->params.empty() ? nullptr : c->params.data(), (int)c->params.size(),
                            c->seed);
        if (rc == DUGKS_OK && !c->out_dir.empty()) rc = snapshot(s, c, s->s_prep, 0);
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
    // group the cases by (model, walls); per group the streaming kernel's items (cases of
    // at least 8 rows) and the tile kernel's tiles (the rest); slot list at the end
    struct Group {
        std::vector<int3> cases;  // (slot, nx, ny) of the streaming kernel
        std::vector<int4> items;
        std::vector<int2> tiles;
    };
    std::map<std::pair<int, int>, Group> groups;
    std::vector<int> slots;
    for (const auto &c : act) {
        const int m = internal::model_of(c->h), w = internal::walls_of(c->h);
        Group &g = groups[{m, w}];
        if (c->grid.ny >= 8) {
            g.cases.push_back(make_int3(c->slot, c->grid.nx, c->grid.ny));
        } else {
            const int nt = f32::batch_tiles_of(c->grid.nx, c->grid.ny);
            for (int t = 0; t < nt; ++t) g.tiles.push_back(make_int2(c->slot, t));
        }
        slots.push_back(c->slot);
    }
    size_t total = 0;
    for (auto &kv : groups) {
        f32::stream_batch_items(kv.second.cases, kv.second.items);
        total += ((kv.second.items.size() * sizeof(int4) + 255) & ~(size_t)255) +
                 ((kv.second.tiles.size() * sizeof(int2) + 255) & ~(size_t)255);
    }
    const size_t slot_off = total;
    total = slot_off + slots.size() * sizeof(int);
    cudaError_t e = cudaMalloc(&ch.dev, total);
    if (e != cudaSuccess) return e;
    std::vector<char> host(total);
    struct Where {
        int model, walls;
        size_t items_off;
        int nitems;
        size_t tiles_off;
        int ntiles;
    };
    std::vector<Where> where;
    size_t off = 0;
    for (auto &kv : groups) {
        Where w{kv.first.first, kv.first.second, off, (int)kv.second.items.size(), 0, (int)kv.second.tiles.size()};
        std::memcpy(host.data() + off, kv.second.items.data(), kv.second.items.size() * sizeof(int4));
        off += (kv.second.items.size() * sizeof(int4) + 255) & ~(size_t)255;
        w.tiles_off = off;
        std::memcpy(host.data() + off, kv.second.tiles.data(), kv.second.tiles.size() * sizeof(int2));
        off += (kv.second.tiles.size() * sizeof(int2) + 255) & ~(size_t)255;
        where.push_back(w);
    }
    std::memcpy(host.data() + slot_off, slots.data(), slots.size() * sizeof(int));
    if ((e = cudaMemcpy(ch.dev, host.data(), total, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
    char *base = static_cast<char *>(ch.dev);
    int64_t launches = 0;
    if ((e = cudaStreamBeginCapture(s->s_batch, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    cudaError_t le = cudaSuccess;
    for (int k = 0; k < s->chunk && le == cudaSuccess; ++k)
        for (const Where &g : where) {
            le = f32::launch_streamb32(g.model, g.walls, reinterpret_cast<const int4 *>(base + g.items_off), g.nitems,
                                       k, s->d_base, s->d_stop, s->s_batch, &launches);
            if (le == cudaSuccess)
                le = f32::launch_batch32(g.model, g.walls, reinterpret_cast<const int2 *>(base + g.tiles_off),
                                         g.ntiles, k, s->d_base, s->d_stop, s->s_batch, &launches);
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

// step number and next stop of a batched case to the device (before the next chunk)
cudaError_t put_steps(dugks_srv *s, const SrvCase &c) {
    s->h_base[c.slot] = (int)c.base;
    s->h_stop[c.slot] = (int)c.dstop;
    cudaError_t e = cudaMemcpyAsync(s->d_base + c.slot, s->h_base + c.slot, sizeof(int), cudaMemcpyHostToDevice,
                                    s->s_batch);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->d_stop + c.slot, s->h_stop + c.slot, sizeof(int), cudaMemcpyHostToDevice, s->s_batch);
    return e;
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
            c->base = internal::steps_done(c->h);
            c->dstop = next_stop(*c, c->base);
            cudaError_t e = f32::batch_set_case(c->slot, P, S, c->base, s->s_batch);
            if (e == cudaSuccess) e = put_steps(s, *c);
            if (e != cudaSuccess) {
                fail_case(s, c, std::string("batch admission: ") + cudaGetErrorString(e), true);
                continue;
            }
            act.push_back(c);
        }
        for (auto &c : leaving) {
            auto it = std::find(act.begin(), act.end(), c);
            if (it != act.end()) act.erase(it);
            if (c->h) finish_case(s, c, s->s_batch, DUGKS_OK);
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
        cudaError_t e;
        {
            TraceRange trace("srv batch chunk");
            e = cudaGraphLaunch(s->graphs[gi].exec, s->s_batch);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s->s_batch);
        }
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
        // advance the host copies of the step numbers; a case at its stop is
        // checked (and written) and either continues or leaves
        std::vector<std::pair<std::shared_ptr<SrvCase>, int>> done;
        for (auto &c : act) {
            c->base += s->chunk;
            if (c->base < c->dstop) {
                std::lock_guard<std::mutex> lk(s->mu);
                c->steps_done = c->base;
                continue;
            }
            // the launches past the stop skipped the case: it is at step dstop
            c->base = c->dstop;
            internal::fp32_adopt_steps(c->h, c->dstop - internal::steps_done(c->h));
            {
                std::lock_guard<std::mutex> lk(s->mu);
                c->steps_done = c->dstop;
            }
            int rc = DUGKS_OK;
            if (at_stop(s, c, s->s_batch, &rc)) {
                done.push_back({c, rc});
                continue;
            }
            c->dstop = next_stop(*c, c->base);
            if (put_steps(s, *c) != cudaSuccess) done.push_back({c, DUGKS_ECUDA});
        }
        for (auto &d : done) {
            act.erase(std::find(act.begin(), act.end(), d.first));
            finish_case(s, d.first, s->s_batch, d.second);
        }
    }
}

// ---- solo lanes
void solo_loop(dugks_srv *s, int lane) {
    cudaSetDevice(s->device);
    cudaStream_t st = s->s_solo[lane];
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
        bool end = false;
        while (rc == DUGKS_OK && !end && !c->cancel && !s->stopping) {
            const int64_t stop = next_stop(*c, c->steps_done);
            if (c->steps_done < stop) {
                const int n = (int)std::min<int64_t>(s->chunk, stop - c->steps_done);
                {
                    TraceRange trace("srv solo chunk");
                    rc = dugks_gpu_step(c->h, n, st);
                    if (rc == DUGKS_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = DUGKS_ECUDA;
                }
                if (rc) break;
                {
                    std::lock_guard<std::mutex> lk(s->mu);
                    c->steps_done += n;
                    s->st.solo_steps += n;
                }
                if (c->steps_done < stop) continue;
            }
            end = at_stop(s, c, st, &rc);
        }
        if (s->stopping) c->cancel = true;
        finish_case(s, c, st, rc);
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
    st->stop_reason = c.stop_reason;
    st->files = c.files;
    st->residual = c.residual;
}

bool terminal(int state) { return state >= DUGKS_SRV_DONE; }

}  // namespace

extern "C" int dugks_srv_create(const dugks_srv_config_t *cfg, dugks_srv_t **out) {
    if (!out) return DUGKS_EINVAL;
    *out = nullptr;
    if (cfg && (cfg->chunk_steps < 0 || cfg->solo_lanes < 0 || cfg->solo_lanes > 64)) return DUGKS_EINVAL;
    auto *s = new (std::nothrow) dugks_srv();
    if (!s) return DUGKS_ENOMEM;
    s->t0 = Clock::now();
    const int lanes = (cfg && cfg->solo_lanes > 0) ? cfg->solo_lanes : 4;
    cudaError_t e = cudaGetDevice(&s->device);
    size_t freeb = 0, totb = 0;
    if (e == cudaSuccess) e = cudaMemGetInfo(&freeb, &totb);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_batch, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->s_prep, cudaStreamNonBlocking);
    for (int k = 0; k < lanes && e == cudaSuccess; ++k) {
        cudaStream_t st = nullptr;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) s->s_solo.push_back(st);
    }
    if (e == cudaSuccess) e = f32::batch_prepare();  // kernel attributes, before any stream capture
    if (e == cudaSuccess) e = cudaMalloc(&s->d_base, 2 * f32::BATCH_MAX_CASES * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_base, 2 * f32::BATCH_MAX_CASES * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(s->d_base, 0, 2 * f32::BATCH_MAX_CASES * sizeof(int));
    if (e != cudaSuccess) {
        dugks_srv_destroy(s);
        return DUGKS_ECUDA;
    }
    s->d_stop = s->d_base + f32::BATCH_MAX_CASES;
    s->h_stop = s->h_base + f32::BATCH_MAX_CASES;
    std::memset(s->h_base, 0, 2 * f32::BATCH_MAX_CASES * sizeof(int));
    s->max_bytes = (cfg && cfg->max_bytes) ? cfg->max_bytes : (size_t)(0.85 * (double)freeb);
    // 50 divides the default check interval (1000 steps), so a batched case
    // never waits out the rest of a chunk at a check
    s->chunk = (cfg && cfg->chunk_steps > 0) ? cfg->chunk_steps : 50;
    s->th_writer = std::thread(writer_loop, s);
    s->th_admit = std::thread(admit_loop, s);
    s->th_batch = std::thread(batch_loop, s);
    for (int k = 0; k < lanes; ++k) s->th_solo.emplace_back(solo_loop, s, k);
    *out = s;
    return DUGKS_OK;
}

extern "C" int dugks_srv_submit_request(dugks_srv_t *s, const dugks_srv_request_t *rq, int64_t *id) {
    if (!s || !rq || !id || rq->nsteps < 0 || rq->nparams < 0 || (rq->nparams > 0 && !rq->params)) return DUGKS_EINVAL;
    if (rq->grid.nx < 3 || rq->grid.ny < 3 || rq->check_every < 0 || rq->snapshot_every < 0 ||
        !(rq->residual_tol >= 0.0))
        return DUGKS_EINVAL;
    if (rq->nsteps > (int64_t)0x7fffffff - 4 * 1024) return DUGKS_EINVAL;  // step numbers are 32-bit on the device
    auto k = std::make_shared<SrvCase>();
    k->cs = rq->cs;
    k->grid = rq->grid;
    k->init_kind = rq->init_kind;
    k->params.assign(rq->params, rq->params + rq->nparams);
    k->seed = rq->seed;
    k->nsteps = rq->nsteps;
    k->residual_tol = rq->residual_tol;
    k->check_every = rq->check_every > 0 ? rq->check_every : DEFAULT_CHECK_EVERY;
    k->snapshot_every = rq->snapshot_every;
    if (rq->out_dir) k->out_dir = rq->out_dir;
    k->bytes = internal::footprint(rq->cs, rq->grid);
    // NEE walls and the UW flux scheme take a solo lane (the batched kernels have the
    // central scheme and bounce-back walls only)
    k->batched = rq->cs.precision == DUGKS_FP32_DEV &&
                 (rq->cs.model == DUGKS_MODEL_AC || rq->cs.model == DUGKS_MODEL_HCZ) &&
                 rq->cs.flux_scheme == DUGKS_FLUX_CD && !(rq->grid.y_walls && rq->cs.wall_scheme == DUGKS_WALL_NEE);
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

extern "C" int dugks_srv_submit(dugks_srv_t *s, const dugks_case_t *c, const dugks_grid_t *g, int init_kind,
                                const double *params, int nparams, uint64_t seed, int64_t nsteps, int64_t *id) {
    if (!c || !g) return DUGKS_EINVAL;
    dugks_srv_request_t rq{};
    rq.cs = *c;
    rq.grid = *g;
    rq.init_kind = init_kind;
    rq.nparams = nparams;
    rq.params = params;
    rq.seed = seed;
    rq.nsteps = nsteps;
    return dugks_srv_submit_request(s, &rq, id);
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
    for (auto &t : s->th_solo)
        if (t.joinable()) t.join();
    // the writer finishes the files of cases that ended
    {
        std::lock_guard<std::mutex> lk(s->wmu);
        s->writer_stop = true;
        s->cv_job.notify_all();
    }
    if (s->th_writer.joinable()) s->th_writer.join();
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
    for (auto &b : s->pinned_all) cudaFreeHost(b.p);
    for (cudaStream_t st : s->s_solo)
        if (st) cudaStreamDestroy(st);
    for (cudaStream_t st : {s->s_batch, s->s_prep})
        if (st) cudaStreamDestroy(st);
    delete s;
    return DUGKS_OK;
}
