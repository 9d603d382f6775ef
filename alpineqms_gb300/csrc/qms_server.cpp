// qms_server.cpp -- native serving object over the qms C-ABI.
//
// A request is one whole solve of the reference program: steady state, then nt
// backward-Euler steps, with the frame velocity of trajectory type 1 and its
// first-step pad (3D/QMS_3D.f90:1428-1449, F:2331-2350), the background field
// optionally scaled by an AC excitation, and the H slice recorded at the
// steady state and every tt steps (the Hx/Hy/Hz.bin cadence, F:1378-1404,
// F:2274-2300).
//
// Scheduling: one admission thread takes requests in arrival order (FIFO, no
// overtaking) and admits the head as soon as its device footprint
// (qms_device_bytes) fits in the budget and a slot is free.  Each admitted
// request runs on its own worker thread with its own qms_handle, hence its own
// CUDA stream: resident solves overlap on the GPU, and a new request starts
// while others are mid-run instead of waiting for a batch to drain.  Results
// are independent of the mix because every reduction is a fixed-order block
// sum.
#include "qms.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

// trajectory type 1: v0 + a n dt while n <= n_acc, v0 + a n_acc dt afterwards (F:2331-2350)
double trajectory_1(double v0, double a, int nacc, int n, double dt) {
    double r = 0.0;
    if (n <= nacc) r = v0 + a * n * dt;
    if (n > nacc) r = v0 + a * nacc * dt;
    return r;
}

// trajectory type 2 (harmonic motion, an extension: the reference stops on it, F:135-151)
double trajectory_2(double amp, double f, double phase, int n, double dt) {
    const double two_pi = 6.283185307179586;   // 2 * pi, rounded to double
    return amp * std::sin(two_pi * f * (n * dt) + phase);
}

// The frame velocity of the steady state and of each step, with the pad of the first
// step: when a dt < v0 * 1E-8 (a default-real literal) the first step accelerates by
// v(0) * 1E-8 / dt (F:1428-1449); the pad state starts at zero (static storage).  The pad
// belongs to type 1 (its test reads that type's a and v0); axes of type 2 (harmonic) and 3
// (a per-step velocity table, the last entry held) get none.
struct VelocitySchedule {
    double tr[3][3];
    int kind[3];
    const double* table[3];
    int len[3];
    double dt;
    double v[3];
    double acc[3] = {0.0, 0.0, 0.0};
    VelocitySchedule(const qms_request& r, const double* const tab[3]) : dt(r.dt) {
        for (int d = 0; d < 3; d++) {
            for (int q = 0; q < 3; q++) tr[d][q] = r.traj[d][q];
            kind[d] = r.traj_kind[d] == 0 ? 1 : r.traj_kind[d];
            table[d] = tab[d];
            len[d] = r.traj_len[d];
            v[d] = velocity(d, 0, 0.0);
        }
    }
    double velocity(int d, int n, double pad) const {
        if (kind[d] == 2) return trajectory_2(tr[d][0], tr[d][1], tr[d][2], n, dt);
        if (kind[d] == 3) return table[d][n < len[d] - 1 ? n : len[d] - 1];
        return trajectory_1(tr[d][0], tr[d][1] + pad, (int)tr[d][2], n, dt);
    }
    void step(int counter, double out[3]) {
        const double eps = (double)1e-8f;
        for (int d = 0; d < 3; d++) {
            if (kind[d] == 1) {
                const double v0 = tr[d][0], a = tr[d][1];
                if (counter == 1) {
                    if (a * dt < v0 * eps) acc[d] = v[d] * eps / dt;
                } else {
                    acc[d] = 0.0;
                }
            }
            out[d] = velocity(d, counter, acc[d]);
        }
        for (int d = 0; d < 3; d++) v[d] = out[d];
    }
};

// Trajectory fields of a request: kinds 0 (= 1), 1, 2 or 3, a table of at least one value for 3.
bool trajectory_ok(const qms_request& r) {
    for (int d = 0; d < 3; d++) {
        const int k = r.traj_kind[d];
        if (k < 0 || k > 3) return false;
        if (k == 3 && (!r.traj_table[d] || r.traj_len[d] < 1)) return false;
    }
    return true;
}

struct Request {
    long long id = 0;
    qms_request r{};                  // scalars; pointers cleared after the copy
    std::vector<double> geom, table;
    std::vector<double> traj_table[3];    // velocity tables of type-3 axes
    size_t footprint = 0;
    int state = QMS_SRV_QUEUED;
    int rc = 0;
    std::string err;
    long long n_dims = 0;
    double arrival = 0, admitted = 0, finished = 0, steady_s = 0;
    std::vector<double> step_s;
    std::vector<double> slices;
};

double percentile(std::vector<double> a, double p) {
    if (a.empty()) return 0.0;
    std::sort(a.begin(), a.end());
    const double pos = p / 100.0 * (double)(a.size() - 1);
    const size_t lo = (size_t)std::floor(pos), hi = std::min(lo + 1, a.size() - 1);
    return a[lo] + (a[hi] - a[lo]) * (pos - (double)lo);
}

}  // namespace

struct qms_server {
    qms_srv_desc d{};
    Clock::time_point t0 = Clock::now();
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Request*> pending;
    std::map<long long, std::unique_ptr<Request>> all;
    std::vector<std::thread> workers;
    std::thread admitter;
    double used = 0.0;
    int resident = 0;
    bool stop = false;
    long long next_id = 0;
    double peak_bytes = 0.0;
    int peak_resident = 0;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

    void admit_loop() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] { return stop || !pending.empty(); });
            if (pending.empty()) {
                if (stop) return;
                continue;
            }
            Request* q = pending.front();       // FIFO: the head waits until it fits
            cv.wait(lk, [&] { return used + (double)q->footprint <= d.budget_bytes && resident < d.max_resident; });
            pending.pop_front();
            used += (double)q->footprint;
            resident++;
            peak_bytes = std::max(peak_bytes, used);
            peak_resident = std::max(peak_resident, resident);
            q->admitted = now();
            q->state = QMS_SRV_RUNNING;
            workers.emplace_back([this, q] { run(q); });
        }
    }

    void fail(Request* q, int rc, const char* what, qms_handle* h) {
        q->rc = rc;
        q->err = std::string(what) + ": " + qms_last_error(h);
    }

    void run(Request* q) {
        const qms_request& r = q->r;
        qms_desc dd;
        qms_default_desc(&dd, r.xs, r.ys, r.zs, r.dx, r.dy, r.dz, r.dt);
        dd.precision = r.precision;
        dd.device = d.device;
        qms_handle* h = nullptr;
        int rc = qms_create(&dd, &h);
        if (rc) {
            fail(q, rc, "qms_create", nullptr);
        } else {
            rc = qms_set_geometry_f64(h, q->geom.data(), q->table.data(), r.nmat);
            if (rc) fail(q, rc, "qms_set_geometry_f64", h);
        }
        if (rc == 0) {
            const int n1 = r.slice_axis == 0 ? r.ys : r.xs, n2 = r.slice_axis == 2 ? r.ys : r.zs;
            const size_t rec = 3 * (size_t)n1 * n2;
            const double* tabs[3] = {q->traj_table[0].data(), q->traj_table[1].data(), q->traj_table[2].data()};
            VelocitySchedule vs(r, tabs);
            auto field = [&](int n, double B[3], double G[9]) {
                const double two_pi = 6.283185307179586;   // 2 * pi, rounded to double
                double s = 1.0;
                const double t = n * r.dt;
                if (r.exc_kind == QMS_EXC_COS) s = std::cos(two_pi * r.exc_f * t + r.exc_phase);
                else if (r.exc_kind == QMS_EXC_SIN) s = std::sin(two_pi * r.exc_f * t + r.exc_phase);
                for (int c = 0; c < 3; c++) B[c] = r.B[c] * s;
                for (int c = 0; c < 9; c++) G[c] = r.G[c] * s;
            };
            auto record = [&]() -> int {
                if (r.keep != QMS_KEEP_SLICES) return 0;
                const size_t at = q->slices.size();
                q->slices.resize(at + rec);
                return qms_get_fields(h, QMS_FIELD_SLICE, r.slice_axis, r.slice_index, q->slices.data() + at);
            };
            double B[3], G[9], v[3];
            field(0, B, G);
            auto t = Clock::now();
            rc = qms_steady(h, vs.v, B, G);
            q->steady_s = std::chrono::duration<double>(Clock::now() - t).count();
            if (rc) fail(q, rc, "qms_steady", h);
            else if ((rc = record())) fail(q, rc, "qms_get_fields", h);
            for (int n = 1; rc == 0 && n <= r.nt; n++) {
                vs.step(n, v);
                field(n, B, G);
                t = Clock::now();
                rc = qms_step(h, v, B, G);
                if (rc) { fail(q, rc, "qms_step", h); break; }
                if (r.tt > 0 && n % r.tt == 0 && (rc = record())) { fail(q, rc, "qms_get_fields", h); break; }
                q->step_s.push_back(std::chrono::duration<double>(Clock::now() - t).count());
            }
        }
        if (h) qms_destroy(h);
        std::lock_guard<std::mutex> lk(mu);
        q->n_dims = qms_n_dims(r.xs, r.ys, r.zs);
        q->finished = now();
        q->state = rc == 0 ? QMS_SRV_DONE : QMS_SRV_FAILED;
        used -= (double)q->footprint;
        resident--;
        cv.notify_all();
    }
};

extern "C" {

int qms_srv_create(const qms_srv_desc* d, qms_server** out) {
    if (!d || !out || !(d->budget_bytes > 0) || d->max_resident < 1) return QMS_ERR_ARG;
    qms_server* s = new (std::nothrow) qms_server();
    if (!s) return QMS_ERR_NOMEM;
    s->d = *d;
    s->admitter = std::thread([s] { s->admit_loop(); });
    *out = s;
    return 0;
}

int qms_srv_submit(qms_server* s, const qms_request* r, long long* id) {
    if (!s || !r || !id || !r->geom || (r->nmat > 0 && !r->table) || r->nmat < 0 || r->nt < 0) return QMS_ERR_ARG;
    if (r->xs < 4 || r->ys < 4 || r->zs < 4 || r->slice_axis < 0 || r->slice_axis > 2 || r->slice_index < 1 ||
        r->slice_index > (r->slice_axis == 0 ? r->xs : r->slice_axis == 1 ? r->ys : r->zs) || !trajectory_ok(*r))
        return QMS_ERR_ARG;
    std::unique_ptr<Request> q(new (std::nothrow) Request());
    if (!q) return QMS_ERR_NOMEM;
    q->r = *r;
    q->geom.assign(r->geom, r->geom + (size_t)r->xs * r->ys * r->zs);
    q->table.assign(r->table, r->table + 7 * (size_t)r->nmat);
    q->r.geom = nullptr;
    q->r.table = nullptr;
    for (int d = 0; d < 3; d++) {
        if (r->traj_kind[d] == 3) q->traj_table[d].assign(r->traj_table[d], r->traj_table[d] + r->traj_len[d]);
        q->r.traj_table[d] = nullptr;
    }
    qms_desc dd;
    qms_default_desc(&dd, r->xs, r->ys, r->zs, r->dx, r->dy, r->dz, r->dt);
    dd.precision = r->precision;
    q->footprint = qms_device_bytes(&dd);
    std::lock_guard<std::mutex> lk(s->mu);
    q->id = s->next_id++;
    q->arrival = s->now();
    if ((double)q->footprint > s->d.budget_bytes) {
        q->state = QMS_SRV_REJECTED;
        q->err = "footprint exceeds the whole budget";
        q->finished = q->arrival;
        q->admitted = q->arrival;
    } else {
        s->pending.push_back(q.get());
    }
    *id = q->id;
    s->all[q->id] = std::move(q);
    s->cv.notify_all();
    return 0;
}

static void fill_result(const Request& q, qms_srv_result* out) {
    out->state = q.state;
    out->rc = q.rc;
    out->n_dims = q.n_dims;
    out->steps_done = (int)q.step_s.size();
    out->arrival_s = q.arrival;
    out->admitted_s = q.admitted;
    out->finished_s = q.finished;
    out->steady_s = q.steady_s;
    double sum = 0.0, mx = 0.0;
    for (double v : q.step_s) { sum += v; mx = std::max(mx, v); }
    out->step_mean_s = q.step_s.empty() ? 0.0 : sum / (double)q.step_s.size();
    out->step_max_s = mx;
    out->n_slice_values = (long long)q.slices.size();
}

int qms_srv_poll(qms_server* s, long long id, qms_srv_result* out) {
    if (!s || !out) return QMS_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return QMS_ERR_ARG;
    fill_result(*it->second, out);
    return 0;
}

int qms_srv_wait(qms_server* s, long long id, qms_srv_result* out) {
    if (!s || !out) return QMS_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return QMS_ERR_ARG;
    Request* q = it->second.get();
    s->cv.wait(lk, [&] { return q->state >= QMS_SRV_DONE; });
    fill_result(*q, out);
    return 0;
}

long long qms_srv_slices(qms_server* s, long long id, double* out, long long cap) {
    if (!s || (cap > 0 && !out) || cap < 0) return QMS_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return QMS_ERR_ARG;
    const Request& q = *it->second;
    if (q.state < QMS_SRV_DONE) return QMS_ERR_STATE;
    const long long n = std::min(cap, (long long)q.slices.size());
    if (n > 0) std::memcpy(out, q.slices.data(), (size_t)n * sizeof(double));
    return n;
}

const char* qms_srv_error(qms_server* s, long long id) {
    if (!s) return "null server";
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return "unknown request id";
    return it->second->err.c_str();
}

int qms_srv_stats_get(qms_server* s, qms_srv_stats* out) {
    if (!s || !out) return QMS_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    qms_srv_stats st{};
    std::vector<double> steps, req, wait;
    double first = -1.0, last = 0.0;
    for (const auto& kv : s->all) {
        const Request& q = *kv.second;
        st.submitted++;
        if (q.state == QMS_SRV_REJECTED) { st.rejected++; continue; }
        if (q.state == QMS_SRV_FAILED) st.failed++;
        if (q.state != QMS_SRV_DONE) continue;
        st.completed++;
        steps.insert(steps.end(), q.step_s.begin(), q.step_s.end());
        req.push_back(q.finished - q.arrival);
        wait.push_back(q.admitted - q.arrival);
        st.dof_timesteps += (double)q.n_dims * (double)q.step_s.size();
        first = first < 0 ? q.arrival : std::min(first, q.arrival);
        last = std::max(last, q.finished);
    }
    st.step_p50_ms = 1e3 * percentile(steps, 50);
    st.step_p99_ms = 1e3 * percentile(steps, 99);
    st.request_p50_s = percentile(req, 50);
    st.request_p99_s = percentile(req, 99);
    st.queue_wait_p50_s = percentile(wait, 50);
    st.queue_wait_p99_s = percentile(wait, 99);
    st.wall_s = first < 0 ? 0.0 : last - first;
    st.peak_bytes = s->peak_bytes;
    st.peak_resident = s->peak_resident;
    *out = st;
    return 0;
}

void qms_srv_destroy(qms_server* s) {
    if (!s) return;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv.notify_all();
    }
    s->admitter.join();                         // returns once every queued request was admitted
    for (auto& t : s->workers) t.join();
    delete s;
}

int qms_srv_velocities(const qms_request* r, int nsteps, double* out) {
    if (!r || !out || nsteps < 0 || !trajectory_ok(*r)) return QMS_ERR_ARG;
    const double* tabs[3] = {r->traj_table[0], r->traj_table[1], r->traj_table[2]};
    VelocitySchedule vs(*r, tabs);
    for (int d = 0; d < 3; d++) out[d] = vs.v[d];
    for (int n = 1; n <= nsteps; n++) vs.step(n, out + 3 * (size_t)n);
    return 0;
}

}  // extern "C"
