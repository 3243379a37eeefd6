// Serving loop: continuous batching of scalar advection-diffusion solves.
//
// Requests (a box mesh, a uniform velocity, a diffusivity and a number of
// implicit steps) arrive at any time through fvgb_server_submit.  A host thread
// admits waiting requests in arrival order whenever their estimated device
// footprint fits the HBM budget, builds their mesh on the device
// (fvgb_mesh_create_boxes) and keeps fields, matrix and solver state resident
// until the request finishes.  Each active request advances on its own CUDA
// stream (from a pool) in chunks of a few time steps; the loop polls the
// chunk-completion events, enqueues the next chunk of every request whose
// previous chunk finished, retires finished requests (copying the result to the
// caller's host buffer) and admits waiting ones as budget frees up, so requests
// of very different sizes progress at their own pace and their work overlaps
// on the GPU.  A request's device memory comes from the server's memory pool
// and goes back to it, in stream order on the request's stream, as soon as its
// result is reported: cudaFree and cudaFreeHost synchronise the whole device,
// and under a saturated stream their flushes idled the GPU for about a second
// every thousand requests.  Each request runs
// exactly the computation it would run alone, so its result does not depend
// on the mix.
//
// Time step (IMEX, as `imp::ddt(T) + exp::div(phi, T) - imp::laplacian(D, T)`):
// explicit upwind convection of the previous field, implicit ddt + diffusion,
// Jacobi-CG (FP64, or mixed precision with an inner reduction of 1e-4 per FP64
// residual replacement) to a relative residual of 1e-8.
// Boundaries: zero gradient; initial field: a Gaussian blob at the box centre.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "fvgb.h"
#include "fvgb_host_common.h"
#include "internal.cuh"

namespace {

using Clock = std::chrono::steady_clock;
constexpr int kChunk = 4;  // steps enqueued per request before the loop looks at it again
constexpr double kServeInnerRelTol = 1e-4;  // mixed precision: inner residual reduction per FP64 replacement

struct Slot {
    int64_t id = 0;
    fvgb_serve_request req{};
    double submit_s = 0, start_s = 0;
    int32_t steps_done = 0, iters = 0, status = FVGB_OK;
    int64_t bytes = 0;
    cudaStream_t stream = nullptr;
    fvgb_mesh* mesh = nullptr;
    fvgb_ls* ls = nullptr;
    int32_t n = 0, nif = 0, nbf = 0;
    double *T = nullptr, *Told = nullptr, *Tb = nullptr, *F = nullptr, *gamma = nullptr, *ref = nullptr;
    double *U = nullptr, *Ub = nullptr;
    fvgb_solver_stats* stats_dev = nullptr;  // [kChunk]
    fvgb_solver_stats* stats_host = nullptr; // pinned [kChunk]
    cudaEvent_t done_ev = nullptr;
    int32_t inflight = 0;                    // steps of the chunk in flight
    int32_t final_status = FVGB_OK;          // set when the request is retiring
    int32_t types[6] = {FVGB_BC_FIXED_GRADIENT, FVGB_BC_FIXED_GRADIENT, FVGB_BC_FIXED_GRADIENT,
                        FVGB_BC_FIXED_GRADIENT, FVGB_BC_FIXED_GRADIENT, FVGB_BC_FIXED_GRADIENT};
    double dt = 0;
};

int64_t nbf_of(const fvgb_serve_request& r) {
    return 2LL * ((int64_t)r.ny * r.nz + (int64_t)r.nx * r.nz + (int64_t)r.nx * r.ny);
}

}  // namespace

struct fvgb_server {
    fvgb_server_cfg cfg{};
    std::vector<cudaStream_t> streams;
    std::thread loop;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Slot*> waiting;
    std::vector<Slot*> active;
    std::vector<fvgb_serve_result> done;
    std::vector<int64_t> cancel_ids;
    int64_t next_id = 1, used = 0, peak_used = 0;
    int64_t ticks = 0;
    bool stop = false;
    int device = 0;
    Clock::time_point t0;
    std::vector<Slot*> retiring;            // result copy enqueued, waiting for its event
    std::vector<fvgb_solver_stats*> free_stats;  // pinned stats buffers of retired requests, reused
    cudaMemPool_t pool = nullptr;           // device memory of the requests (devmem_*)
    cudaStream_t alloc_stream = nullptr;    // the pool's allocation stream

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Device bytes a request holds while resident (mesh, system, solver, fields).
int64_t estimate_bytes(const fvgb_serve_request& r) {
    const int64_t n = ((int64_t)r.nx * r.ny * r.nz + 31) / 32 * 32;
    const int64_t nif = (int64_t)(r.nx - 1) * r.ny * r.nz + (int64_t)r.nx * (r.ny - 1) * r.nz +
                        (int64_t)r.nx * r.ny * (r.nz - 1);
    const int64_t nbf = nbf_of(r);
    const int64_t mesh = 16 * n + 72 * nif + 64 * nbf + 4 * 6 * 2 * n + 4 * 7 * 2 * n + 2 * 7 * n + 4 * n;
    const int64_t system = 8 * 7 * n + 8 * n + 16 * nbf;
    const int64_t solver = r.precision == FVGB_PREC_MIXED_IR ? (8 + 28 + 16) * n : 40 * n;
    const int64_t fields = 16 * n + 8 * nbf + 16 * (nif + nbf) + 24 * (n + nbf) + 8 * nbf;
    return mesh + system + solver + fields + (1 << 20);
}

// Device memory of a request comes from the server's pool (set on the loop's
// thread, devmem_*) and is released in stream order on the request's stream:
// no device synchronisation.  Its pinned stats buffer goes back to the server's
// free list (cudaFreeHost would synchronise the device).
void release(fvgb_server* sv, Slot* s) {
    devmem_ctx().release = s->stream;
    double* bufs[] = {s->T, s->Told, s->Tb, s->F, s->gamma, s->ref, s->U, s->Ub};
    for (double* b : bufs) devmem_free(b, true);
    devmem_free(s->stats_dev, true);
    if (s->stats_host) sv->free_stats.push_back(s->stats_host);
    if (s->done_ev) cudaEventDestroy(s->done_ev);
    s->stats_host = nullptr;
    s->done_ev = nullptr;
    if (s->ls) fvgb_ls_destroy(s->ls);
    if (s->mesh) fvgb_mesh_destroy(s->mesh);
    s->T = s->Told = s->Tb = s->F = s->gamma = s->ref = s->U = s->Ub = nullptr;
    s->stats_dev = nullptr;
    s->ls = nullptr;
    s->mesh = nullptr;
    devmem_ctx().release = nullptr;
}

__global__ void k_blob(double* T, int nx, int ny, int nz, int cell0) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nx * ny * nz) return;
    const int i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
    const double x = (i + 0.5) / nx - 0.5, y = (j + 0.5) / ny - 0.5, z = (k + 0.5) / nz - 0.5;
    T[cell0 + c] = exp(-(x * x + y * y + z * z) / (2.0 * 0.1 * 0.1));
}

__global__ void k_fill3(double* a, int count, double x, double y, double z) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= count) return;
    a[3 * c] = x;
    a[3 * c + 1] = y;
    a[3 * c + 2] = z;
}

__global__ void k_fill(double* a, int count, double v) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < count) a[c] = v;
}

fvgb_status setup(fvgb_server* sv, Slot* s) {
    const fvgb_serve_request& r = s->req;
    fvgb_box_spec spec{r.nx, r.ny, r.nz, 1.0, 1.0, 1.0, 0.0, 0, 0};
    int32_t range[2];
    fvgb_status st = fvgb_mesh_create_boxes(&spec, 1, &s->mesh, range, s->stream);
    if (st != FVGB_OK) return st;
    int64_t sz[5];
    fvgb_mesh_sizes(s->mesh, sz);
    s->n = (int32_t)sz[0];
    s->nif = (int32_t)sz[1];
    s->nbf = (int32_t)sz[2];
    st = fvgb_ls_create(s->mesh, 1, &s->ls);
    if (st != FVGB_OK) return st;
    const size_t n = (size_t)s->n, nbf = (size_t)s->nbf, nf = (size_t)(s->nif + s->nbf);
    cudaError_t e = cudaSuccess;
    auto A = [&](double** p, size_t count) {
        if (e == cudaSuccess) e = devmem_alloc((void**)p, sizeof(double) * (count ? count : 1), true);
    };
    A(&s->T, n);
    if (r.flags & FVGB_SERVE_REASSEMBLE) A(&s->Told, n);
    A(&s->Tb, nbf);
    A(&s->F, nf);
    A(&s->gamma, nf);
    A(&s->ref, nbf);
    A(&s->U, 3 * n);
    A(&s->Ub, 3 * nbf);
    if (e == cudaSuccess) e = devmem_alloc((void**)&s->stats_dev, sizeof(fvgb_solver_stats) * kChunk, true);
    if (e == cudaSuccess) {
        if (!sv->free_stats.empty()) {
            s->stats_host = sv->free_stats.back();
            sv->free_stats.pop_back();
        } else {
            e = cudaMallocHost(&s->stats_host, sizeof(fvgb_solver_stats) * kChunk);
        }
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->done_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) return fvgb_fail(FVGB_ERR_OOM, "server: request allocation");
    const int nn = s->n, rn = r.nx * r.ny * r.nz;
    k_fill<<<(nn + 255) / 256, 256, 0, s->stream>>>(s->T, nn, 0.0);
    if (r.T_init) {
        if (cudaMemcpyAsync(s->T + range[0], r.T_init, sizeof(double) * (size_t)rn, cudaMemcpyHostToDevice,
                            s->stream) != cudaSuccess)
            return fvgb_fail(FVGB_ERR_CUDA, "server: initial field upload");
    } else {
        k_blob<<<(rn + 255) / 256, 256, 0, s->stream>>>(s->T, r.nx, r.ny, r.nz, range[0]);
    }
    k_fill<<<(int)((nbf + 255) / 256 + 1), 256, 0, s->stream>>>(s->ref, (int)nbf, 0.0);
    k_fill<<<(int)((nf + 255) / 256), 256, 0, s->stream>>>(s->gamma, (int)nf, r.D);
    k_fill3<<<(nn + 255) / 256, 256, 0, s->stream>>>(s->U, nn, r.U[0], r.U[1], r.U[2]);
    k_fill3<<<(int)((nbf + 255) / 256 + 1), 256, 0, s->stream>>>(s->Ub, (int)nbf, r.U[0], r.U[1], r.U[2]);
    fvgb_bc bc{s->types, s->ref};
    st = fvgb_bc_correct(s->mesh, 1, &bc, s->T, s->Tb, s->stream);
    if (st == FVGB_OK) st = fvgb_flux_vec(s->mesh, s->U, s->Ub, s->F, s->stream);
    if (st != FVGB_OK) return st;
    const double umag = std::sqrt(r.U[0] * r.U[0] + r.U[1] * r.U[1] + r.U[2] * r.U[2]);
    const double h = 1.0 / std::max(r.nx, std::max(r.ny, r.nz));
    s->dt = r.dt > 0 ? r.dt : 0.5 * h / std::max(umag, 1e-12);
    (void)sv;
    return FVGB_OK;
}

fvgb_status enqueue_step(Slot* s, int k) {
    const fvgb_serve_request& r = s->req;
    // The old field: the reference's pattern (FVGB_SERVE_REASSEMBLE) keeps a copy of
    // it, as NeoN's oldTime field is stored every step.  Otherwise it is T itself:
    // the assembly reads it before the solve overwrites T (its initial guess) in
    // place, so no copy is needed.  Same values, same bits.
    const double* old = s->T;
    if (r.flags & FVGB_SERVE_REASSEMBLE) {
        if (cudaMemcpyAsync(s->Told, s->T, sizeof(double) * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream) !=
            cudaSuccess)
            return fvgb_fail(FVGB_ERR_CUDA, "server: copy");
        old = s->Told;
    }
    fvgb_term terms[3] = {
        {FVGB_TERM_DDT, 0, 1.0, old, nullptr},
        {FVGB_TERM_DIV_EXPLICIT, FVGB_SCHEME_UPWIND, 1.0, old, s->F},
        {FVGB_TERM_LAPLACIAN, 0, -1.0, nullptr, s->gamma},
    };
    fvgb_bc bc{s->types, s->ref};
    // the implicit part (ddt + diffusion) is the same every step: after the first
    // step only the rhs is assembled, and the solve keeps its FP32 matrix copy
    const bool full = s->steps_done + k == 0 || (r.flags & FVGB_SERVE_REASSEMBLE);
    fvgb_status st = full ? fvgb_assemble(s->ls, terms, 3, s->dt, &bc, s->Tb, s->stream)
                          : fvgb_assemble_rhs(s->ls, terms, 3, s->dt, &bc, s->Tb, s->stream);
    if (st != FVGB_OK) return st;
    // the graph path by default: requests overlap on the device, which one
    // cooperative (persistent) kernel per request would serialise.  Mixed
    // precision: a warm-started step needs about 7 CG iterations, so the FP64
    // residual replacements set its cost; an inner reduction of 1e-4 needs two
    // of them to reach 1e-8 where 0.1 needs eight (served stream of 2,000
    // requests: 58.6 solves/s against 45.3, FP64 56.9)
    fvgb_solver_cfg cfg{1e-8, 0.0, 2000, r.precision, kServeInnerRelTol, 1000, 50,
                        r.kernel_mode == 0 ? 1 : r.kernel_mode,
                        FVGB_SOLVE_NO_TUNE};  // tuning would synchronise the device under every request
    st = fvgb_solve_async(s->ls, s->T, &cfg, s->stats_dev + k, s->stream);
    if (st != FVGB_OK) return st;
    return fvgb_bc_correct(s->mesh, 1, &bc, s->T, s->Tb, s->stream);
}

void report(fvgb_server* sv, Slot* s);

// Enqueue the result copy and an event after it; the loop reports the request
// once the event has completed (no stream synchronisation in the loop).
void finish(fvgb_server* sv, Slot* s, int32_t status) {
    if (status == FVGB_OK && s->req.T_out && s->mesh) {
        // the box occupies rows [0, nx*ny*nz) of its own mesh
        const size_t rn = (size_t)s->req.nx * s->req.ny * s->req.nz;
        cudaMemcpyAsync(s->req.T_out, s->T, sizeof(double) * rn, cudaMemcpyDeviceToHost, s->stream);
    }
    s->final_status = status;
    if (s->stream && s->done_ev && cudaEventRecord(s->done_ev, s->stream) == cudaSuccess) {
        sv->retiring.push_back(s);
        return;
    }
    if (s->stream) cudaStreamSynchronize(s->stream);
    report(sv, s);
}

// The request's result is in the caller's buffer: publish it.
void report(fvgb_server* sv, Slot* s) {
    const int32_t status = s->final_status;
    fvgb_serve_result res{};
    res.id = s->id;
    res.status = status;
    res.steps_done = s->steps_done;
    res.total_iters = s->iters;
    res.submit_s = s->submit_s;
    res.start_s = s->start_s;
    res.finish_s = sv->now();
    res.device_bytes = s->bytes;
    // the request's work has completed (its event): its memory goes back to
    // the pool now, and its budget with it
    release(sv, s);
    const int64_t bytes = s->bytes;
    delete s;
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->used -= bytes;
    sv->done.push_back(res);
}

// The requests' device memory pool: kept across releases (no release
// threshold), and reused only once a release has executed, never by making a
// later allocation wait on another request's stream.
void open_pool(fvgb_server* sv) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = sv->device;
    if (cudaMemPoolCreate(&sv->pool, &props) != cudaSuccess) {
        cudaGetLastError();
        sv->pool = nullptr;
        cudaDeviceGetDefaultMemPool(&sv->pool, sv->device);
    }
    uint64_t keep = ~0ull;
    int no = 0;
    cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    cudaMemPoolSetAttribute(sv->pool, cudaMemPoolReuseAllowInternalDependencies, &no);
    cudaStreamCreateWithFlags(&sv->alloc_stream, cudaStreamNonBlocking);
    devmem_ctx() = DevMemCtx{sv->pool, sv->alloc_stream, nullptr};
}

void close_pool(fvgb_server* sv) {
    cudaDeviceSynchronize();  // every release has executed
    for (fvgb_solver_stats* p : sv->free_stats) cudaFreeHost(p);
    sv->free_stats.clear();
    cudaMemPool_t dflt = nullptr;
    cudaDeviceGetDefaultMemPool(&dflt, sv->device);
    if (sv->pool && sv->pool != dflt) cudaMemPoolDestroy(sv->pool);
    if (sv->alloc_stream) cudaStreamDestroy(sv->alloc_stream);
    sv->pool = nullptr;
    sv->alloc_stream = nullptr;
    devmem_ctx() = DevMemCtx{};
}

void run(fvgb_server* sv) {
    cudaSetDevice(sv->device);
    open_pool(sv);
    size_t next_stream = 0;
    for (;;) {
        std::vector<Slot*> admit;
        std::vector<int64_t> cancels;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv.wait(lk, [&] {
                return sv->stop || !sv->waiting.empty() || !sv->active.empty() || !sv->retiring.empty();
            });
            if (sv->stop && sv->waiting.empty() && sv->active.empty() && sv->retiring.empty()) break;
            cancels.swap(sv->cancel_ids);
            // cancel waiting requests
            for (auto it = sv->waiting.begin(); it != sv->waiting.end();) {
                if (std::find(cancels.begin(), cancels.end(), (*it)->id) != cancels.end()) {
                    fvgb_serve_result res{};
                    res.id = (*it)->id;
                    res.status = FVGB_ERR_CANCELLED;
                    res.submit_s = (*it)->submit_s;
                    res.finish_s = sv->now();
                    sv->done.push_back(res);
                    delete *it;
                    it = sv->waiting.erase(it);
                } else {
                    ++it;
                }
            }
            // admit in arrival order while the head fits the budget
            while (!sv->waiting.empty() && (int32_t)(sv->active.size() + admit.size()) < sv->cfg.max_active) {
                Slot* s = sv->waiting.front();
                if (sv->used + s->bytes > sv->cfg.budget_bytes) break;
                sv->used += s->bytes;
                sv->peak_used = std::max(sv->peak_used, sv->used);
                sv->waiting.pop_front();
                admit.push_back(s);
            }
        }
        for (Slot* s : admit) {
            s->stream = sv->streams[next_stream++ % sv->streams.size()];
            s->start_s = sv->now();
            fvgb_status st = setup(sv, s);
            if (st != FVGB_OK) {
                finish(sv, s, st);
                continue;
            }
            sv->active.push_back(s);
        }
        // cancel active requests between steps
        if (!cancels.empty()) {
            std::vector<Slot*> keep;
            for (Slot* s : sv->active) {
                if (std::find(cancels.begin(), cancels.end(), s->id) != cancels.end()) finish(sv, s, FVGB_ERR_CANCELLED);
                else keep.push_back(s);
            }
            sv->active.swap(keep);
        }
        // publish requests whose result copy has completed
        bool progressed = !admit.empty();
        {
            std::vector<Slot*> still;
            for (Slot* s : sv->retiring) {
                if (cudaEventQuery(s->done_ev) == cudaErrorNotReady) {
                    still.push_back(s);
                } else {
                    report(sv, s);
                    progressed = true;
                }
            }
            sv->retiring.swap(still);
        }
        // advance every request whose previous chunk finished
        std::vector<Slot*> keep;
        for (Slot* s : sv->active) {
            if (s->inflight > 0) {
                const cudaError_t q = cudaEventQuery(s->done_ev);
                if (q == cudaErrorNotReady) {
                    keep.push_back(s);
                    continue;
                }
                progressed = true;
                int32_t status = q == cudaSuccess ? FVGB_OK : FVGB_ERR_CUDA;
                for (int k = 0; k < s->inflight && status == FVGB_OK; ++k) {
                    s->iters += s->stats_host[k].num_iter;
                    s->steps_done += 1;
                    if (s->stats_host[k].status != FVGB_OK) status = s->stats_host[k].status;
                }
                s->inflight = 0;
                if (status != FVGB_OK || s->steps_done >= s->req.steps) {
                    finish(sv, s, status);
                    continue;
                }
            }
            const int todo = std::min(kChunk, s->req.steps - s->steps_done);
            int32_t status = FVGB_OK;
            for (int k = 0; k < todo && status == FVGB_OK; ++k) status = enqueue_step(s, k);
            if (status == FVGB_OK &&
                cudaMemcpyAsync(s->stats_host, s->stats_dev, sizeof(fvgb_solver_stats) * todo,
                                cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
                status = FVGB_ERR_CUDA;
            if (status == FVGB_OK && cudaEventRecord(s->done_ev, s->stream) != cudaSuccess) status = FVGB_ERR_CUDA;
            if (status != FVGB_OK) {
                finish(sv, s, status);
                continue;
            }
            s->inflight = todo;
            progressed = true;
            keep.push_back(s);
        }
        sv->active.swap(keep);
        ++sv->ticks;
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    close_pool(sv);
}

}  // namespace

extern "C" fvgb_status fvgb_server_create(const fvgb_server_cfg* cfg, fvgb_server** out) {
    fvgb_clear_error();
    if (!cfg || !out || cfg->budget_bytes <= 0 || cfg->n_streams <= 0 || cfg->n_streams > 64 || cfg->max_active <= 0)
        return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_server_create: bad configuration");
    fvgb_server* sv = new fvgb_server();
    sv->cfg = *cfg;
    sv->t0 = Clock::now();
    cudaGetDevice(&sv->device);
    for (int i = 0; i < cfg->n_streams; ++i) {
        cudaStream_t s;
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
            for (cudaStream_t t : sv->streams) cudaStreamDestroy(t);
            delete sv;
            return fvgb_fail(FVGB_ERR_CUDA, "fvgb_server_create: stream creation");
        }
        sv->streams.push_back(s);
    }
    sv->loop = std::thread(run, sv);
    *out = sv;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_server_submit(fvgb_server* sv, const fvgb_serve_request* req, int64_t* id) {
    if (!sv || !req || !id) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_server_submit: null argument");
    if (req->nx < 2 || req->ny < 2 || req->nz < 2 || req->steps < 1 || !(req->D >= 0) ||
        (req->precision != FVGB_PREC_FP64 && req->precision != FVGB_PREC_MIXED_IR) || req->kernel_mode < 0 ||
        req->kernel_mode > 3 || (req->kernel_mode == 3 && req->precision != FVGB_PREC_FP64))
        return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_server_submit: bad request");
    Slot* s = new Slot();
    s->req = *req;
    s->bytes = estimate_bytes(*req);
    if (s->bytes > sv->cfg.budget_bytes) {
        delete s;
        return fvgb_fail(FVGB_ERR_BUDGET, "fvgb_server_submit: request alone exceeds the HBM budget");
    }
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stop) {
            delete s;
            return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_server_submit: server is shutting down");
        }
        s->id = sv->next_id++;
        s->submit_s = sv->now();
        sv->waiting.push_back(s);
        *id = s->id;
    }
    sv->cv.notify_one();
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_server_cancel(fvgb_server* sv, int64_t id) {
    if (!sv) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_server_cancel: null server");
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->cancel_ids.push_back(id);
    }
    sv->cv.notify_one();
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_server_poll(fvgb_server* sv, fvgb_serve_result* out, int32_t max, int32_t* count) {
    if (!sv || !count || (max > 0 && !out)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_server_poll: bad argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    const int32_t k = std::min<int32_t>(max, (int32_t)sv->done.size());
    for (int32_t i = 0; i < k; ++i) out[i] = sv->done[i];
    sv->done.erase(sv->done.begin(), sv->done.begin() + k);
    *count = k;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_server_info(fvgb_server* sv, int64_t out[6]) {
    if (!sv || !out) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_server_info: bad argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    out[0] = (int64_t)sv->waiting.size();
    out[1] = (int64_t)sv->active.size();
    out[2] = (int64_t)sv->done.size();
    out[3] = sv->used;
    out[4] = sv->peak_used;
    out[5] = sv->ticks;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_server_destroy(fvgb_server* sv) {
    if (!sv) return FVGB_OK;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv.notify_one();
    if (sv->loop.joinable()) sv->loop.join();
    for (cudaStream_t s : sv->streams) cudaStreamDestroy(s);
    delete sv;
    return FVGB_OK;
}
