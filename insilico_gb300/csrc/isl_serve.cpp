// Served Newton solves with continuous batching (isl_serve_*).
//
// The reference runs one boundary-value problem at a time through
// solid::CompressibleDriver (solid/CompressibleDriver.hpp:156-214): per load
// step it scales the constraints by (k+1)/k, then iterates Newton: assemble
// the tangent and the residual, stop when ||R||/N < tol, solve, add the
// increment to the DOFs, stop when ||dU||/N < tol.
//
// Here a server admits many such requests and runs them on one GPU:
//   * a scheduler thread forms batches from the queue in arrival order (or,
//     with order = 1, starting from the largest queued request):
//     requests with the same element shape, components, kernel, material and
//     quadrature (and, with size_ratio > 1, element counts within that factor
//     of the batch's first request), up to max_batch, within the 32-bit
//     contribution budget of a context and within the free HBM
//     (cudaMemGetInfo) minus a reserve;
//   * each batch is one isl_ctx holding its requests as instances
//     (isl_batch_mesh_upload) on its own CUDA stream and host thread, so
//     batches formed from later arrivals run concurrently with earlier ones
//     and a batch's memory returns to the pool as soon as it finishes;
//   * inside a batch every Newton iteration is shared: one assembly launch
//     sequence over all instances' elements, one device reduction for all
//     instances' ||R||/N (isl_batch_norms), one batched CG in which every
//     instance keeps its own scalars and convergence, one distribute.  The
//     instances' Newton loops run the reference's logic independently on the
//     host from the per-instance norms: an instance whose load step has
//     converged moves to its next step (isl_batch_scale_constraints) while
//     the others keep iterating; isl_batch_set_mask keeps instances that need
//     no solve in this iteration out of the solve and the distribute;
//   * a finished request's displacement is copied out and its ticket
//     completes while its batch runs on.
// A batch of one runs the same batched kernels, so a request's result does
// not depend on what it was batched with (bit for bit).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "isl_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

int nverts(int shape) { return shape == ISL_QUAD ? 4 : shape == ISL_TET ? 4 : 8; }
int sdim(int shape) { return shape == ISL_QUAD ? 2 : 3; }

struct Req {
    int64_t ticket = 0;
    // copied inputs
    int shape = 0, ncomp = 0, kernel = 0, material = 0, qdeg = 0;
    int64_t n_nodes = 0, n_elem = 0;
    std::vector<double> X, coef0, coef1, body;
    std::vector<int64_t> conn, fnode;
    std::vector<int> fcomp;
    std::vector<double> fval;
    int load_steps = 1, max_newton = 1;
    double tol = 0.0, lin_tol = 1e-10;
    // state and results
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
    int status = ISL_OK;
    std::string err;
    std::vector<double> u;
    int64_t newton = 0, cg = 0, steps_done = 0, batch_id = -1;
    int batch_size = 0;
    bool converged = true;
    double t_submit = 0, t_admit = 0, t_finish = 0;
    int64_t footprint = 0, pairs = 0;
};

struct Batch {
    int64_t id = 0;
    std::vector<std::shared_ptr<Req>> reqs;
    int64_t footprint = 0;
};

}  // namespace

struct isl_server {
    int device = 0;
    isl_serve_config cfg{};
    Clock::time_point t0 = Clock::now();
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::shared_ptr<Req>> queue;
    std::map<int64_t, std::shared_ptr<Req>> reqs;
    struct Worker {
        std::thread t;
        std::shared_ptr<std::atomic<bool>> done;
    };
    std::vector<Worker> workers;
    int running = 0;
    int64_t reserved = 0;  // footprints of running batches
    int64_t launches = 0;  // kernel launches of finished batches
    // host wall time of the finished batches: setup, assembly (+ norms),
    // solve (+ distribute, norms), whole batch; Newton iterations run
    double t_setup = 0, t_assemble = 0, t_solve = 0, t_batches = 0;
    int64_t ticks = 0;
    int64_t next_ticket = 1, next_batch = 0;
    bool stop = false;
    std::thread sched;
    std::string err;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

// Peak device memory of a request (pattern build included), from its size:
// element pairs (n_elem * nloc^2) bound the contributions and the nonzeros.
void estimate(Req& r) {
    const int nloc = nverts(r.shape) * r.ncomp;
    r.pairs = r.n_elem * (int64_t)nloc * nloc;
    const int64_t nup = (int64_t)nloc * (nloc + 1) / 2;
    const int64_t neq = r.n_nodes * r.ncomp;
    const int64_t nnz = std::min<int64_t>(r.pairs, neq * (int64_t)nloc * 4);
    const int64_t persistent = nnz * (4 + 4 + 8 + 4 + 4 + 4) + r.pairs * 4 + r.n_elem * nup * 8 + neq * 160 +
                               r.n_nodes * 8 * (sdim(r.shape) + r.ncomp);
    r.footprint = persistent + r.pairs * 24;
}

int64_t free_bytes(isl_server* s) {
    if (s->cfg.test_budget_bytes > 0) return s->cfg.test_budget_bytes - s->reserved;
    int64_t f = 0, t = 0;
    if (isl_device_memory(s->device, &f, &t) != ISL_OK) return 0;
    // reservations count in full: part of them is already allocated and
    // visible in the free figure, so this errs on the safe side
    return f - s->reserved;
}

bool same_kind(const Req& a, const Req& b) {
    return a.shape == b.shape && a.ncomp == b.ncomp && a.kernel == b.kernel && a.material == b.material &&
           a.qdeg == b.qdeg && a.lin_tol == b.lin_tol;
}

void finish_req(isl_server* s, Req& r, int state) {
    std::lock_guard<std::mutex> lk(s->mu);
    r.state = state;
    r.t_finish = s->now();
    s->cv.notify_all();
}

void fail_batch(isl_server* s, Batch& b, int status, const std::string& msg) {
    for (auto& r : b.reqs) {
        if (r->state >= 2) continue;
        r->status = status;
        r->err = msg;
        finish_req(s, *r, 3);
    }
}

#define SV_CHECK(call)                                                             \
    do {                                                                           \
        const int _st = (call);                                                    \
        if (_st != ISL_OK) {                                                       \
            fail_batch(s, b, _st, std::string(#call) + ": " + isl_last_error(c)); \
            return;                                                                \
        }                                                                          \
    } while (0)

// Simulated work for scheduler tests without a GPU: every request finishes
// after one pass, taking fake_us_per_elem microseconds per element of its batch.
void run_fake(isl_server* s, Batch& b) {
    int64_t ne = 0;
    for (auto& r : b.reqs) ne += r->n_elem;
    std::this_thread::sleep_for(std::chrono::microseconds((int64_t)(s->cfg.test_fake_us_per_elem * ne)));
    for (auto& r : b.reqs) {
        r->u.assign((size_t)r->n_nodes * r->ncomp, 0.0);
        r->newton = 1;
        r->steps_done = r->load_steps;
        finish_req(s, *r, 2);
    }
}

// One batch: setup of the batched context, then the Newton iterations of all
// its requests in shared launches (see the file comment).
void run_batch(isl_server* s, Batch& b) {
    const double t_begin = std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
    const int n = (int)b.reqs.size();
    const Req& r0 = *b.reqs[0];
    const int dim = sdim(r0.shape), nv = nverts(r0.shape), nc = r0.ncomp;
    isl_ctx* c = nullptr;
    if (isl_ctx_create(&c, s->device, nullptr) != ISL_OK) {
        fail_batch(s, b, ISL_ERR_CUDA, "isl_ctx_create failed");
        return;
    }
    struct Guard {
        isl_server* s;
        isl_ctx* c;
        ~Guard() {
            int64_t n = 0;
            if (isl_launch_count(c, &n) == ISL_OK) {
                std::lock_guard<std::mutex> lk(s->mu);
                s->launches += n;
            }
            isl_ctx_destroy(c);
        }
    } guard{s, c};
    // concatenated instances
    std::vector<int64_t> node_off(n + 1, 0), elem_off(n + 1, 0);
    for (int k = 0; k < n; ++k) {
        node_off[k + 1] = node_off[k] + b.reqs[k]->n_nodes;
        elem_off[k + 1] = elem_off[k] + b.reqs[k]->n_elem;
    }
    std::vector<double> X((size_t)node_off[n] * dim), c0((size_t)elem_off[n]), c1;
    std::vector<int64_t> conn((size_t)elem_off[n] * nv);
    bool body = false;
    for (auto& r : b.reqs) body |= !r->body.empty();
    std::vector<double> fb(body ? (size_t)node_off[n] * nc : 0, 0.0);
    if (r0.kernel == ISL_KERNEL_HYPERELASTIC) c1.resize((size_t)elem_off[n]);
    for (int k = 0; k < n; ++k) {
        const Req& r = *b.reqs[k];
        std::copy(r.X.begin(), r.X.end(), X.begin() + node_off[k] * dim);
        for (size_t i = 0; i < r.conn.size(); ++i) conn[(size_t)elem_off[k] * nv + i] = r.conn[i] + node_off[k];
        std::copy(r.coef0.begin(), r.coef0.end(), c0.begin() + elem_off[k]);
        if (!c1.empty()) std::copy(r.coef1.begin(), r.coef1.end(), c1.begin() + elem_off[k]);
        if (body && !r.body.empty()) std::copy(r.body.begin(), r.body.end(), fb.begin() + node_off[k] * nc);
    }
    SV_CHECK(isl_batch_mesh_upload(c, r0.shape, dim, n, node_off.data(), X.data(), elem_off.data(), conn.data()));
    int64_t ndofobj = 0;
    int nfun = 0;
    SV_CHECK(isl_field_create(c, 1, nc, &ndofobj, &nfun));
    // Dirichlet values of the first load step; an isoparametric field has one
    // DOF object per node
    {
        std::vector<int64_t> obj;
        std::vector<int> comp;
        std::vector<double> val;
        for (int k = 0; k < n; ++k) {
            const Req& r = *b.reqs[k];
            for (size_t i = 0; i < r.fnode.size(); ++i) {
                obj.push_back(node_off[k] + r.fnode[i]);
                comp.push_back(r.fcomp[i]);
                val.push_back(r.fval[i]);
            }
        }
        if (!obj.empty()) SV_CHECK(isl_constrain(c, (int64_t)obj.size(), obj.data(), comp.data(), val.data()));
    }
    int64_t neq = 0, nnz = 0;
    SV_CHECK(isl_number_dofs(c, &neq));
    SV_CHECK(isl_register_pattern(c, &nnz));
    if (r0.kernel == ISL_KERNEL_LAPLACE) SV_CHECK(isl_set_laplace(c, c0.data(), r0.qdeg));
    else SV_CHECK(isl_set_hyperelastic(c, r0.material, c0.data(), c1.data(), r0.qdeg));
    if (body) SV_CHECK(isl_set_body_force_nodal(c, fb.data()));
    // a batching server runs the batched solver for every batch size, with a
    // fixed FP32 SpMV kind (per-instance reductions in a fixed order: results
    // independent of the batch); a server of one request per batch runs the
    // single-system solvers
    const bool batched = s->cfg.max_batch > 1;
    if (batched) {
        SV_CHECK(isl_set_option(c, ISL_OPT_BATCHED_SOLVE, 1));
        if (s->cfg.precision != ISL_PREC_FP64) SV_CHECK(isl_set_option(c, ISL_OPT_SPMV32_KIND, 104));
    } else {
        // a one-launch solve of a small system holds every SM (cooperative
        // grid) and would serialise the batches that run at the same time
        SV_CHECK(isl_set_option(c, ISL_OPT_PERSISTENT, s->cfg.persistent == 1 ? 1 : 0));
    }
    std::vector<int64_t> eq_off(n + 1), dof_off(n + 1);
    int64_t ninst = 0;
    SV_CHECK(isl_batch_info(c, &ninst, eq_off.data(), dof_off.data()));

    const int prec = s->cfg.precision;
    const int method = prec == ISL_PREC_FP64 ? ISL_SOLVE_CG_FP64 : ISL_SOLVE_CG_FP32_IR;
    // per-instance Newton state (solid/CompressibleDriver.hpp:156-214)
    std::vector<int> step(n, 0), iter(n, 0), active(n, 1);
    std::vector<double> factor(n, 1.0), normR(n), normDU(n);
    std::vector<uint8_t> solve(n, 0);
    std::vector<int64_t> cgit(n);
    std::vector<double> relres(n), uall((size_t)ndofobj * nc);
    const double lin_tol = r0.lin_tol;  // the same in a batch
    int nactive = n;
    int64_t max_ticks = 4;
    for (auto& r : b.reqs) max_ticks = std::max<int64_t>(max_ticks, (int64_t)r->load_steps * (r->max_newton + 1) + 4);

    // instance k's load step is over: the next one scales its constraints
    // by (k+1)/k (CompressibleDriver.hpp:164-172), or the request is done
    auto next_step = [&](int k, std::vector<int>& done_now) {
        ++step[k];
        iter[k] = 0;
        if (step[k] >= b.reqs[k]->load_steps) done_now.push_back(k);
        else factor[k] = (double)(step[k] + 1) / (double)step[k];
    };

    double t_asm = 0.0, t_solve = 0.0;
    int64_t ticks = 0;
    auto stamp = [] { return std::chrono::duration<double>(Clock::now().time_since_epoch()).count(); };
    const double t_setup = stamp() - t_begin;
    struct Account {  // the batch's phase times go to the server's totals however the loop ends
        isl_server* s;
        const double &setup, &as, &so;
        const int64_t& ticks;
        double t0;
        ~Account() {
            const double tot = std::chrono::duration<double>(Clock::now().time_since_epoch()).count() - t0;
            std::lock_guard<std::mutex> lk(s->mu);
            s->t_setup += setup;
            s->t_assemble += as;
            s->t_solve += so;
            s->t_batches += tot;
            s->ticks += ticks;
        }
    } account{s, t_setup, t_asm, t_solve, ticks, t_begin};
    for (int64_t tick = 0; nactive > 0; ++tick) {
        ++ticks;
        if (tick > max_ticks) {  // cannot happen: every iteration advances an instance
            fail_batch(s, b, ISL_ERR_TIMEOUT, "served Newton loop made no progress");
            return;
        }
        // scale the constraints of instances that start a new load step
        bool scale = false;
        for (int k = 0; k < n; ++k) scale |= factor[k] != 1.0;
        if (scale) {
            SV_CHECK(isl_batch_scale_constraints(c, factor.data()));
            std::fill(factor.begin(), factor.end(), 1.0);
        }
        double t0 = stamp();
        SV_CHECK(isl_assemble(c, prec, 1, 1));
        SV_CHECK(isl_batch_norms(c, normR.data()));
        t_asm += stamp() - t0;
        std::vector<int> done_now;
        int nsolve = 0;
        for (int k = 0; k < n; ++k) {
            solve[k] = 0;
            if (!active[k]) continue;
            if (normR[k] < b.reqs[k]->tol) { next_step(k, done_now); continue; }
            solve[k] = 1;
            ++nsolve;
        }
        if (nsolve > 0) {
            t0 = stamp();
            if (n > 1) SV_CHECK(isl_batch_set_mask(c, solve.data()));
            int64_t it = 0;
            double rr = 0.0;
            const int st = isl_solve(c, method, lin_tol, 0, &it, &rr);
            // an inexact Newton step may stop at its iteration limit
            if (st != ISL_OK && st != ISL_ERR_NOT_CONVERGED) {
                fail_batch(s, b, st, std::string("isl_solve: ") + isl_last_error(c));
                return;
            }
            if (batched) SV_CHECK(isl_batch_solve_stats(c, cgit.data(), relres.data()));
            else cgit[0] = it;
            SV_CHECK(isl_distribute(c, 1));
            SV_CHECK(isl_batch_norms(c, normDU.data()));
            t_solve += stamp() - t0;
            for (int k = 0; k < n; ++k) {
                if (!solve[k]) continue;
                Req& r = *b.reqs[k];
                r.cg += cgit[k];
                ++r.newton;
                ++iter[k];
                const bool conv = normDU[k] < r.tol;
                if (!conv && iter[k] >= r.max_newton) r.converged = false;
                if (conv || iter[k] >= r.max_newton) next_step(k, done_now);
            }
        }
        if (!done_now.empty()) {
            // finished instances: copy their DOF values out, complete their tickets
            SV_CHECK(isl_get_values(c, uall.data()));
            for (int k : done_now) {
                Req& r = *b.reqs[k];
                r.u.assign(uall.begin() + dof_off[k] * nc, uall.begin() + dof_off[k + 1] * nc);
                r.steps_done = step[k];
                finish_req(s, r, 2);
                active[k] = 0;
                --nactive;
            }
        }
    }
}

void worker_main(isl_server* s, std::shared_ptr<Batch> b, std::shared_ptr<std::atomic<bool>> done) {
    if (s->cfg.test_fake_us_per_elem > 0) run_fake(s, *b);
    else {
        cudaSetDevice(s->device);
        run_batch(s, *b);
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->running--;
        s->reserved -= b->footprint;
        s->cv.notify_all();
    }
    done->store(true);
}

// Forms batches from the queue in arrival order and starts them while the
// batch limit and the free HBM allow (a batch that finds the GPU idle is
// admitted whatever its size, so an oversized request still runs alone).
void scheduler_main(isl_server* s) {
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv.wait(lk, [&] { return s->stop || (!s->queue.empty() && s->running < s->cfg.max_batches); });
        if (s->stop && s->queue.empty()) break;
        if (s->stop) {  // destroy with requests still queued: they fail
            for (auto& r : s->queue) {
                r->status = ISL_ERR_ARG;
                r->err = "server destroyed before the request ran";
                r->state = 3;
                r->t_finish = s->now();
            }
            s->queue.clear();
            s->cv.notify_all();
            break;
        }
        // join the threads of finished batches
        for (auto it = s->workers.begin(); it != s->workers.end();) {
            if (it->done->load()) {
                it->t.join();
                it = s->workers.erase(it);
            } else {
                ++it;
            }
        }
        // batching window: a partial batch waits for more arrivals until its
        // oldest request has queued for batch_window_us
        if (s->cfg.batch_window_us > 0 && (int)s->queue.size() < s->cfg.max_batch && !s->stop) {
            const double waited = s->now() - s->queue.front()->t_submit;
            const double window = 1e-6 * (double)s->cfg.batch_window_us;
            if (waited < window) {
                s->cv.wait_for(lk, std::chrono::duration<double>(window - waited));
                continue;
            }
        }
        if (s->cfg.order == 1 && s->queue.size() > 1) {
            // largest first: the first of the largest requests leads the batch
            auto big = std::max_element(s->queue.begin(), s->queue.end(),
                                        [](const std::shared_ptr<Req>& a, const std::shared_ptr<Req>& b) {
                                            return a->n_elem < b->n_elem;
                                        });
            if (big != s->queue.begin()) {
                auto r = *big;
                s->queue.erase(big);
                s->queue.push_front(r);
            }
        }
        auto b = std::make_shared<Batch>();
        const int64_t avail = free_bytes(s) - s->cfg.reserve_bytes;
        int64_t pairs = 0;
        for (auto it = s->queue.begin(); it != s->queue.end() && (int)b->reqs.size() < s->cfg.max_batch;) {
            Req& r = **it;
            const bool first = b->reqs.empty();
            if (!first && !same_kind(r, *b->reqs[0])) { ++it; continue; }
            if (!first && s->cfg.size_ratio > 1.0) {
                const double h = (double)b->reqs[0]->n_elem, e = (double)r.n_elem;
                if (e > h * s->cfg.size_ratio || e * s->cfg.size_ratio < h) { ++it; continue; }
            }
            const bool fits_mem = b->footprint + r.footprint <= avail;
            const bool fits_pairs = pairs + r.pairs <= s->cfg.max_pairs;
            if (first ? (fits_mem || s->running == 0) : (fits_mem && fits_pairs)) {
                b->reqs.push_back(*it);
                b->footprint += r.footprint;
                pairs += r.pairs;
                it = s->queue.erase(it);
            } else if (first) {
                break;  // the head of the queue waits for memory
            } else {
                ++it;
            }
        }
        if (b->reqs.empty()) {  // not enough memory yet: wait for a batch to finish
            s->cv.wait_for(lk, std::chrono::milliseconds(5));
            continue;
        }
        b->id = s->next_batch++;
        const double t = s->now();
        for (auto& r : b->reqs) {
            r->batch_id = b->id;
            r->batch_size = (int)b->reqs.size();
            r->state = 1;
            r->t_admit = t;
        }
        s->running++;
        s->reserved += b->footprint;
        auto done = std::make_shared<std::atomic<bool>>(false);
        s->workers.push_back({std::thread(worker_main, s, b, done), done});
    }
}

}  // namespace

extern "C" {

int isl_serve_create(isl_server** out, int device, const isl_serve_config* cfg) {
    ISL_TRY
    if (!out || !cfg) return ISL_ERR_ARG;
    *out = nullptr;
    if (cfg->max_batch < 1 || cfg->max_batches < 1) return ISL_ERR_ARG;
    if (cfg->precision < ISL_PREC_FP64 || cfg->precision > ISL_PREC_MIXED) return ISL_ERR_ARG;
    if (cfg->test_fake_us_per_elem <= 0) {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return ISL_ERR_ARG;
    }
    auto* s = new isl_server();
    s->device = device;
    s->cfg = *cfg;
    if (s->cfg.max_pairs <= 0) s->cfg.max_pairs = 1300000000LL;  // 32-bit contribution lists
    s->sched = std::thread(scheduler_main, s);
    *out = s;
    return ISL_OK;
    ISL_CATCH(nullptr)
}

int isl_serve_submit(isl_server* s, const isl_serve_request* q, int64_t* ticket) {
    ISL_TRY
    if (!s || !q || !ticket) return ISL_ERR_ARG;
    const int nv = (q->shape == ISL_QUAD || q->shape == ISL_TET || q->shape == ISL_HEX) ? nverts(q->shape) : 0;
    if (!nv || q->n_nodes <= 0 || q->n_elem <= 0 || !q->coords || !q->conn || !q->coef0) return ISL_ERR_ARG;
    const int dim = sdim(q->shape);
    if (q->kernel == ISL_KERNEL_LAPLACE) {
        if (q->ncomp != 1) return ISL_ERR_ARG;
    } else if (q->kernel == ISL_KERNEL_HYPERELASTIC) {
        if (q->ncomp != dim || !q->coef1 || (q->material != ISL_MAT_STVENANT && q->material != ISL_MAT_NEOHOOKE))
            return ISL_ERR_ARG;
    } else {
        return ISL_ERR_ARG;
    }
    if (q->load_steps < 1 || q->max_newton < 1 || !(q->tolerance >= 0.0) || !(q->lin_tol > 0.0)) return ISL_ERR_ARG;
    if (q->n_fixed < 0 || (q->n_fixed > 0 && (!q->fixed_node || !q->fixed_comp || !q->fixed_value))) return ISL_ERR_ARG;
    auto r = std::make_shared<Req>();
    r->shape = q->shape; r->ncomp = q->ncomp; r->kernel = q->kernel; r->material = q->material;
    r->qdeg = q->quad_degree; r->n_nodes = q->n_nodes; r->n_elem = q->n_elem;
    r->X.assign(q->coords, q->coords + q->n_nodes * dim);
    r->conn.assign(q->conn, q->conn + q->n_elem * nv);
    for (int64_t v : r->conn) if (v < 0 || v >= q->n_nodes) return ISL_ERR_ARG;
    r->coef0.assign(q->coef0, q->coef0 + q->n_elem);
    if (q->kernel == ISL_KERNEL_HYPERELASTIC) r->coef1.assign(q->coef1, q->coef1 + q->n_elem);
    if (q->body) r->body.assign(q->body, q->body + q->n_nodes * q->ncomp);
    r->fnode.assign(q->fixed_node, q->fixed_node + q->n_fixed);
    r->fcomp.assign(q->fixed_comp, q->fixed_comp + q->n_fixed);
    r->fval.assign(q->fixed_value, q->fixed_value + q->n_fixed);
    for (int64_t i = 0; i < q->n_fixed; ++i)
        if (r->fnode[i] < 0 || r->fnode[i] >= q->n_nodes || r->fcomp[i] < 0 || r->fcomp[i] >= q->ncomp) return ISL_ERR_ARG;
    r->load_steps = q->load_steps; r->max_newton = q->max_newton;
    r->tol = q->tolerance; r->lin_tol = q->lin_tol;
    estimate(*r);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return ISL_ERR_ARG;
    r->ticket = s->next_ticket++;
    r->t_submit = s->now();
    s->reqs[r->ticket] = r;
    s->queue.push_back(r);
    *ticket = r->ticket;
    s->cv.notify_all();
    return ISL_OK;
    ISL_CATCH(nullptr)
}

int isl_serve_poll(isl_server* s, int64_t ticket, int* state) {
    if (!s || !state) return ISL_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return ISL_ERR_ARG;
    *state = it->second->state;
    return ISL_OK;
}

int isl_serve_wait(isl_server* s, int64_t ticket, double timeout_s, int* state) {
    ISL_TRY
    if (!s || !state) return ISL_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return ISL_ERR_ARG;
    auto r = it->second;
    s->cv.wait_for(lk, std::chrono::duration<double>(std::max(0.0, timeout_s)), [&] { return r->state >= 2; });
    *state = r->state;
    return r->state >= 2 ? ISL_OK : ISL_ERR_TIMEOUT;
    ISL_CATCH(nullptr)
}

int isl_serve_result(isl_server* s, int64_t ticket, double* u, isl_serve_stats* st) {
    ISL_TRY
    if (!s) return ISL_ERR_ARG;
    std::shared_ptr<Req> r;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(ticket);
        if (it == s->reqs.end()) return ISL_ERR_ARG;
        r = it->second;
        if (r->state < 2) return ISL_ERR_ARG;
    }
    if (st) {
        st->newton_iters = r->newton;
        st->cg_iters = r->cg;
        st->load_steps_done = r->steps_done;
        st->converged = r->converged && r->state == 2;
        st->status = r->status;
        st->t_submit = r->t_submit;
        st->t_admit = r->t_admit;
        st->t_finish = r->t_finish;
        st->batch_id = r->batch_id;
        st->batch_size = r->batch_size;
    }
    if (u && r->state == 2) std::copy(r->u.begin(), r->u.end(), u);
    return r->state == 2 ? ISL_OK : r->status;
    ISL_CATCH(nullptr)
}

const char* isl_serve_error(isl_server* s, int64_t ticket) {
    if (!s) return "no server";
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return "unknown ticket";
    return it->second->err.c_str();
}

int isl_serve_times(isl_server* s, double* setup_s, double* assemble_s, double* solve_s, double* batch_s,
                    int64_t* newton_ticks) {
    if (!s) return ISL_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (setup_s) *setup_s = s->t_setup;
    if (assemble_s) *assemble_s = s->t_assemble;
    if (solve_s) *solve_s = s->t_solve;
    if (batch_s) *batch_s = s->t_batches;
    if (newton_ticks) *newton_ticks = s->ticks;
    return ISL_OK;
}

int isl_serve_counters(isl_server* s, int64_t* launches, int64_t* batches) {
    if (!s) return ISL_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (launches) *launches = s->launches;
    if (batches) *batches = s->next_batch;
    return ISL_OK;
}

int isl_serve_release(isl_server* s, int64_t ticket) {
    if (!s) return ISL_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end() || it->second->state < 2) return ISL_ERR_ARG;
    s->reqs.erase(it);
    return ISL_OK;
}

int isl_serve_destroy(isl_server* s) {
    if (!s) return ISL_ERR_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    s->sched.join();
    for (auto& w : s->workers) w.t.join();
    delete s;
    return ISL_OK;
}

}  // extern "C"
