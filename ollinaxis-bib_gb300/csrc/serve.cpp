// Request loop over evolutions: continuous batching on one GPU.
//
// The reference runs one evolution per process (src/base/evolve.f90); there
// is nothing to mirror here but its per-evolution sequence, which each
// admitted request follows: initial data (``initial``, with its elliptic
// solve), ``initialize`` (evolve.f90:128-219), an initial maximal-slicing
// solve where evolve.f90:228-230 makes one, then ``onestep(0)`` per coarse
// step with the solves of :388-393, and at the end the 0-D norms of
// save0Ddata.f90:221-288.
//
// Design (one host thread, one stream per evolution):
//   * admission by device bytes: a request's footprint (resident while it
//     runs, plus what its elliptic solves add while they run) must fit in the
//     budget beside the resident bytes of the running evolutions;
//   * every running evolution keeps one coarse step queued on its stream;
//     a step that has finished is followed at once by the next, without
//     waiting for the other evolutions, so grids of different sizes keep
//     the GPU filled together; the set-up of newly admitted requests runs on
//     their own streams beside the queued steps;
//   * nothing is shared between evolutions on the device, so a result does
//     not depend on which other requests ran beside it;
//   * small grids make a coarse step a few hundred short kernels, so issuing
//     them binds the loop: the steps of different evolutions are issued from
//     several host threads at once (each evolution from one thread at a time;
//     a handle's state is touched by no one else meanwhile).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ollin_gpu.h"

namespace {

thread_local std::string s_err;

int sfail(int code, const std::string& msg) {
    s_err = msg;
    return code;
}

struct Request {
    long long id = 0;
    ollin_params p{};
    int nsteps = 0;           // coarse steps to the end time
    double collapse = 0.0;    // smallest-lapse threshold (0: none)
    int maximalevery = 0;     // param maximalevery
    size_t resident = 0, transient = 0;
    double t_submit = 0.0;
};

struct Running {
    Request r;
    ollin_handle* h = nullptr;
    double t_admit = 0.0, t_ready = 0.0;
    int steps = 0;
    double t = 0.0;
    double min_alpha = 1.0;
    bool queued = false;  // a step_begin waits for its step_end
    int begin_rc = OLLIN_OK;
};

int min_lapse(ollin_handle* h, double* out_min) { return ollin_gpu_min_lapse(h, out_min); }

// Host threads that run one job per index; the calling thread takes part.
class Workers {
  public:
    explicit Workers(int n) {
        for (int k = 0; k < n; ++k) th_.emplace_back([this] { loop(); });
    }
    ~Workers() {
        {
            std::lock_guard<std::mutex> g(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (std::thread& t : th_) t.join();
    }
    // f(0) .. f(n-1), each once; returns when all have returned
    void run(int n, const std::function<void(int)>& f) {
        if (n <= 0) return;
        std::unique_lock<std::mutex> g(m_);
        job_ = &f;
        n_ = n;
        next_ = 0;
        left_ = n;
        ++gen_;
        cv_.notify_all();
        work(g);
        done_.wait(g, [this] { return left_ == 0; });
        job_ = nullptr;
    }

  private:
    // takes and runs indices until none is left (called with the lock held)
    void work(std::unique_lock<std::mutex>& g) {
        while (job_ && next_ < n_) {
            const int k = next_++;
            const std::function<void(int)>* f = job_;
            g.unlock();
            (*f)(k);
            g.lock();
            if (--left_ == 0) done_.notify_all();
        }
    }
    void loop() {
        std::unique_lock<std::mutex> g(m_);
        unsigned long seen = gen_;
        for (;;) {
            cv_.wait(g, [&] { return stop_ || gen_ != seen; });
            if (stop_) return;
            seen = gen_;
            work(g);
        }
    }
    std::vector<std::thread> th_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    const std::function<void(int)>* job_ = nullptr;
    int n_ = 0, next_ = 0, left_ = 0;
    unsigned long gen_ = 0;
    bool stop_ = false;
};

bool maximal_at_start(const Request& r) {  // evolve.f90:228-230
    return r.p.slicing == OLLIN_SLICING_MAXIMAL || r.p.ilapse == OLLIN_ILAPSE_MAXIMAL || r.maximalevery != 0;
}

bool maximal_after(const Request& r, int step) {  // evolve.f90:388-393
    return r.p.slicing == OLLIN_SLICING_MAXIMAL || (r.maximalevery != 0 && step % r.maximalevery == 0);
}

}  // namespace

struct ollin_server {
    size_t budget = 0;
    int max_active = 1;
    size_t used = 0, peak = 0;
    std::deque<Request> waiting;
    std::vector<Running> running;
    std::deque<ollin_result> done;
    std::chrono::steady_clock::time_point t0;
    Workers* workers = nullptr;  // issue threads besides the caller's
    int graphs = 1;              // coarse steps as captured graphs (ollin_gpu_step_graphs)
    int fused = 0;               // 1: each tick is one fused coarse step of every running evolution

    double now() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    ollin_result result_of(const Request& r, int status) const {
        ollin_result x{};
        x.id = r.id;
        x.status = status;
        x.t_submit = r.t_submit;
        x.bytes = r.resident + r.transient;
        x.min_alpha = NAN;
        return x;
    }

    // ends a running evolution: final norms, then the handle goes
    void retire(size_t k, int status, bool collapsed) {
        Running& e = running[k];
        if (e.queued) {  // its queued work finishes before the handle goes
            double t;
            ollin_gpu_step_end(e.h, &t);
            e.queued = false;
        }
        ollin_result x = result_of(e.r, status);
        x.t_admit = e.t_admit;
        x.t_ready = e.t_ready;
        x.collapsed = collapsed ? 1 : 0;
        x.steps = e.steps;
        x.t = e.t;
        x.min_alpha = e.min_alpha;
        x.ngrids = ollin_gpu_num_levels(e.h);
        x.point_updates = ollin_gpu_point_updates(e.h);
        if (status == OLLIN_OK) {
            static const int fields[4] = {OLLIN_F_ALPHA, OLLIN_F_PHI, OLLIN_F_TRK, OLLIN_F_HAM};
            for (int l = 0; l < std::min(x.ngrids, OLLIN_RESULT_MAXGRIDS) && x.status == OLLIN_OK; ++l)
                for (int f = 0; f < 4; ++f) {
                    double nm[5];
                    int rc = ollin_gpu_norms(e.h, l, fields[f], nm);
                    if (rc) { x.status = rc; break; }
                    x.l2[l][f] = nm[3];
                }
            if (x.status == OLLIN_OK && e.r.collapse <= 0.0) {
                double m;
                if (min_lapse(e.h, &m) == OLLIN_OK) x.min_alpha = m;
            }
        }
        ollin_gpu_destroy(e.h);
        x.t_done = now();
        used -= e.r.resident;
        done.push_back(x);
        running.erase(running.begin() + (long)k);
    }

    // create, initial data, initialize and the first maximal solve of one
    // request, queued on its own stream
    int start(Request& r, Running& e) {
        int rc = ollin_gpu_create(&r.p, &e.h);
        if (rc) { e.h = nullptr; return rc; }
        ollin_gpu_step_graphs(e.h, graphs, nullptr);
        // evolutions side by side fill the SMs themselves; a chained
        // successor's blocks waiting on an SM would only take room from them
        ollin_gpu_step_chaining(e.h, 0);
        rc = ollin_gpu_initial_data(e.h);
        if (!rc) rc = ollin_gpu_initialize(e.h);
        if (!rc && maximal_at_start(r)) rc = ollin_gpu_maximal_slicing(e.h, nullptr);
        if (!rc && r.collapse > 0.0) rc = min_lapse(e.h, &e.min_alpha);
        return rc;
    }

    void admit() {
        for (auto it = waiting.begin(); it != waiting.end() && (int)running.size() < max_active;) {
            if (used + it->resident + it->transient > budget) { ++it; continue; }  // first fit
            Request r = *it;
            it = waiting.erase(it);
            Running e;
            e.r = r;
            e.t_admit = now();
            used += r.resident;
            peak = std::max(peak, used + r.transient);
            int rc = start(r, e);
            if (rc) {
                if (e.h) ollin_gpu_destroy(e.h);
                used -= r.resident;
                ollin_result x = result_of(r, rc);
                x.t_admit = e.t_admit;
                x.t_done = now();
                done.push_back(x);
                continue;
            }
            e.t_ready = now();
            running.push_back(e);
        }
    }
};

extern "C" {

int ollin_server_create(size_t budget, int max_active, ollin_server** out) {
    if (!out || max_active < 1) return sfail(OLLIN_EINVAL, "bad argument");
    auto* s = new ollin_server();
    s->budget = budget;
    s->max_active = max_active;
    s->t0 = std::chrono::steady_clock::now();
    const int hw = (int)std::thread::hardware_concurrency();
    const int nthreads = std::max(0, std::min({hw > 0 ? hw : 1, max_active, 8}) - 1);
    s->workers = new Workers(nthreads);
    *out = s;
    return OLLIN_OK;
}

void ollin_server_destroy(ollin_server* s) {
    if (!s) return;
    while (!s->running.empty()) s->retire(s->running.size() - 1, OLLIN_ESTATE, false);
    delete s->workers;
    delete s;
}

int ollin_server_submit(ollin_server* s, long long id, const ollin_params* p, int maximalevery, double t_end,
                        double collapse_alpha) {
    if (!s || !p || !(t_end >= 0.0) || maximalevery < 0) return sfail(OLLIN_EINVAL, "bad argument");
    Request r;
    r.id = id;
    r.p = *p;
    r.collapse = collapse_alpha;
    r.maximalevery = maximalevery;
    r.t_submit = s->now();
    int rc = ollin_gpu_footprint(p, &r.resident, &r.transient);
    if (rc) return sfail(rc, ollin_gpu_last_error());
    if (r.resident + r.transient > s->budget) return sfail(OLLIN_ENOMEM, "the request can never fit the device budget");
    const double dt0 = p->dtfac * std::min(p->dr0, p->dz0);  // setupboxes.f90:121-125
    r.nsteps = (int)std::ceil(t_end / dt0 - 1e-9);
    s->waiting.push_back(r);
    return OLLIN_OK;
}

namespace {

// A tick of the fused schedule: one coarse step of every running evolution,
// each kernel of the step issued once for all of them
// (ollin_gpu_coarse_step_fused), then each evolution's end-of-step work and
// the admissions.  Requests admitted now join the next tick's step.
int fused_tick(ollin_server* s) {
    const size_t nrun = s->running.size();
    if (nrun > 0) {
        std::vector<ollin_handle*> hs(nrun);
        for (size_t k = 0; k < nrun; ++k) hs[k] = s->running[k].h;
        std::vector<double> t(nrun, 0.0);
        std::vector<int> st(nrun, OLLIN_OK);
        const int rc_all = ollin_gpu_coarse_step_fused(hs.data(), (int)nrun, t.data(), st.data());
        std::vector<int> rc(nrun, OLLIN_OK);
        std::vector<char> coll(nrun, 0), fin(nrun, 0);
        s->workers->run((int)nrun, [&](int q) {
            const size_t k = (size_t)q;
            Running& e = s->running[k];
            // a failure outside any one evolution's flag ends them all
            int r = st[k] ? st[k] : (rc_all && rc_all != OLLIN_ENAN ? rc_all : OLLIN_OK);
            if (!r) { e.t = t[k]; e.steps += 1; }
            if (!r && maximal_after(e.r, e.steps)) r = ollin_gpu_maximal_slicing(e.h, nullptr);
            if (!r && e.r.collapse > 0.0) {
                r = min_lapse(e.h, &e.min_alpha);
                coll[k] = !r && e.min_alpha < e.r.collapse;
            }
            rc[k] = r;
            fin[k] = r || coll[k] || e.steps >= e.r.nsteps;
        });
        for (size_t q = nrun; q-- > 0;)
            if (fin[q]) s->retire(q, rc[q], coll[q] != 0);
    }
    s->admit();
    return OLLIN_OK;
}

}  // namespace

int ollin_server_set_fused(ollin_server* s, int enable) {
    if (!s) return sfail(OLLIN_EINVAL, "null server");
    for (const Running& e : s->running)
        if (e.queued) return sfail(OLLIN_ESTATE, "the schedule changes only when no step is queued");
    s->fused = enable != 0;
    return OLLIN_OK;
}

int ollin_server_tick(ollin_server* s, int* n_active, int* n_waiting) {
    if (!s) return sfail(OLLIN_EINVAL, "null server");
    if (s->fused) {
        const int rc = fused_tick(s);
        if (n_active) *n_active = (int)s->running.size();
        if (n_waiting) *n_waiting = (int)s->waiting.size();
        return rc;
    }
    for (int spin = 0;; ++spin) {
        // (1) every evolution whose step finished: the step's end, the solve
        //     that follows it, the checks, then its next step
        const size_t nrun = s->running.size();
        std::vector<int> rc(nrun, OLLIN_OK);
        std::vector<char> coll(nrun, 0), fin(nrun, 0), moved(nrun, 0);
        std::vector<int> ready;  // found on this thread: waking the others costs more than a query
        for (size_t k = 0; k < nrun; ++k)
            if (!s->running[k].queued || ollin_gpu_step_ready(s->running[k].h)) ready.push_back((int)k);
        s->workers->run((int)ready.size(), [&](int q) {
            const int k = ready[(size_t)q];
            Running& e = s->running[(size_t)k];
            if (e.queued) {
                double t = e.t;
                int r = ollin_gpu_step_end(e.h, &t);
                e.queued = false;
                if (e.begin_rc) r = e.begin_rc;
                if (!r) { e.t = t; e.steps += 1; }
                if (!r && maximal_after(e.r, e.steps)) r = ollin_gpu_maximal_slicing(e.h, nullptr);
                if (!r && e.r.collapse > 0.0) {
                    r = min_lapse(e.h, &e.min_alpha);
                    coll[(size_t)k] = !r && e.min_alpha < e.r.collapse;
                }
                rc[(size_t)k] = r;
            }
            moved[(size_t)k] = 1;
            if (rc[(size_t)k] || coll[(size_t)k] || e.steps >= e.r.nsteps) { fin[(size_t)k] = 1; return; }
            e.begin_rc = ollin_gpu_step_begin(e.h);
            e.queued = true;
        });
        bool progressed = false;
        for (size_t q = nrun; q-- > 0;) {
            progressed = progressed || moved[q];
            if (fin[q]) s->retire(q, rc[q], coll[q] != 0);
        }
        // (2) admissions: their set-up overlaps the queued steps
        const size_t before = s->running.size() + s->done.size();
        s->admit();
        progressed = progressed || s->running.size() + s->done.size() != before;
        if (progressed || s->running.empty()) break;
        // nothing finished yet: wait a little for the queued steps
        if (spin > 64) std::this_thread::sleep_for(std::chrono::microseconds(20));
        else std::this_thread::yield();
    }
    if (n_active) *n_active = (int)s->running.size();
    if (n_waiting) *n_waiting = (int)s->waiting.size();
    return OLLIN_OK;
}

int ollin_server_poll(ollin_server* s, ollin_result* out, int max, int* n_out) {
    if (!s || (!out && max > 0) || !n_out) return sfail(OLLIN_EINVAL, "bad argument");
    int n = 0;
    while (n < max && !s->done.empty()) {
        out[n++] = s->done.front();
        s->done.pop_front();
    }
    *n_out = n;
    return OLLIN_OK;
}

int ollin_server_set_graphs(ollin_server* s, int enable) {
    if (!s) return sfail(OLLIN_EINVAL, "null server");
    s->graphs = enable != 0;
    return OLLIN_OK;
}

int ollin_server_usage(const ollin_server* s, size_t* used, size_t* peak) {
    if (!s || !used || !peak) return sfail(OLLIN_EINVAL, "bad argument");
    *used = s->used;
    *peak = s->peak;
    return OLLIN_OK;
}

const char* ollin_server_last_error(void) { return s_err.c_str(); }

}  // extern "C"
