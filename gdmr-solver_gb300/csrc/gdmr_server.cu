// Serving layer of libgDMR: resident operators, HBM-budget admission and continuous
// batching of solve requests (gdmr_server_* in gdmr_ext.h).
//
// The reference solves one right-hand side per solverDMR call (gDMR.cu:2638-2900) and
// keeps one deflation space per process.  Here every registered operator keeps its matrix
// and its recycled deflation space resident, and owns an engine of `capacity` slots, a
// stream and a worker thread.  A worker admits queued requests into free slots between
// restart cycles, runs one FP64-refined cycle for every request in flight, and hands
// finished solutions back; requests of different operators run on different streams and
// overlap on the device.  The device memory of all engines is fixed at registration and
// bounded by the server's budget, which is what admission by HBM budget means here.
//
// A server may span several devices (independent operators shard across GPUs with no
// collective: §8(e) of the design; the reference instead splits one basis across devices with
// peer copies, gDMR.cu:1478-1520).  Each device of the server's list has its own budget, and
// gdmr_server_add_operator places an operator, with its matrix, its deflation space, its
// engine and its queue, on the device that keeps the most budget free after taking it
// (worst fit, which balances memory and so the work across devices).  A device may appear
// twice in the list (two budgets on one GPU), as the reference's device lists allow.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gdmr_engine.h"

extern "C" {
#include "../../include/gdmr_ext.h"
}

using namespace gdmr;
using Clock = std::chrono::steady_clock;

namespace {

struct Request {
    long long ticket = 0;
    const double *b = nullptr;     // caller's host buffer, n interleaved complex128
    double *x = nullptr;           // caller's host buffer for the solution
    double tol = 1e-10;
    int max_cycles = 0;
    Clock::time_point t_submit;
};

struct Done {
    long long ticket;
    gdmr_stats stats;
};

struct ServedOperator {
    int id = 0, n = 0, m = 0, k = 0, capacity = 0, precision = 1, device = 0;
    int slot_dev = 0;              // index of the server's device (budget) list it was placed on
    DeviceSell A;
    Engine<float> e32;
    Engine<double> e64;
    cudaStream_t st = nullptr;
    double2 *stage = nullptr;      // capacity vectors: H2D staging of right-hand sides
    double *pinned_b = nullptr;    // pinned host staging, capacity vectors
    double *pinned_x = nullptr;
    std::deque<Request> queue;
    std::vector<Request> slot_req;
    std::vector<bool> slot_busy;
    std::thread worker;
    long long bytes = 0;
    // frees everything it holds, also after a registration that failed part of the way (the
    // worker thread, if any, has been joined)
    ~ServedOperator() {
        cudaSetDevice(device);
        if (st) cudaStreamSynchronize(st);
        e32.release();
        e64.release();
        sell_free(A);
        if (stage) cudaFree(stage);
        if (pinned_b) cudaFreeHost(pinned_b);
        if (pinned_x) cudaFreeHost(pinned_x);
        if (st) cudaStreamDestroy(st);
    }
};

}  // namespace

struct gdmr_server {
    long long budget = 0, used = 0;            // totals over the devices
    int device = 0;                           // the first device of the list
    std::vector<int> devices;                 // CUDA ordinals, one per budget
    std::vector<long long> dev_budget, dev_used;
    std::vector<std::unique_ptr<ServedOperator>> ops;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<Done> finished;
    std::unordered_map<long long, gdmr_stats> results;
    std::atomic<bool> running{false};
    std::atomic<long long> next_ticket{1};
    std::atomic<int> errors{0};
    std::string error;
};

namespace {

size_t slot_bytes(int n, int m, int precision) {
    const size_t s = precision == 1 ? sizeof(float2) : sizeof(double2);
    // basis (m+1) + R, X, Y, T in the inner precision; b, x, r in FP64; staging (1)
    return (size_t)n * (s * (m + 1 + 4) + sizeof(double2) * 4);
}

size_t fixed_bytes(int n, int m, int k, int precision, long padded) {
    const size_t s = precision == 1 ? sizeof(float2) : sizeof(double2);
    const size_t matrix = (size_t)padded * (sizeof(int) + sizeof(double2) + (precision == 1 ? sizeof(float2) : 0));
    return matrix + (size_t)n * s * (3 * std::max(k, 1) + 1) + (size_t)(m + 1) * m * 64 + (64u << 20);
}

template <class R> Engine<R> &engine(ServedOperator &op);
template <> Engine<float> &engine<float>(ServedOperator &op) { return op.e32; }
template <> Engine<double> &engine<double>(ServedOperator &op) { return op.e64; }

void fill_stats(const SolveStats &s, gdmr_stats *o) {
    o->cycles = s.cycles;
    o->its = s.its;
    o->matvecs = s.matvecs;
    o->rel_res = s.rel_res;
    o->true_rel_res = s.true_rel_res;
    o->status = s.status;
    o->breakdowns = s.breakdowns;
    o->latency_ms = 0;
}

template <class R> void worker_loop(gdmr_server *srv, ServedOperator *op) {
    cudaSetDevice(op->device);
    Engine<R> &E = engine<R>(*op);
    const size_t vb = sizeof(double2) * (size_t)op->n;
    if (E.refine_setup(op->A.view64()) != GDMR_OK) {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->errors++;
        srv->error = last_error();
        return;
    }
    while (true) {
        // admit queued requests into free slots
        std::vector<std::pair<int, Request>> admit;
        {
            std::unique_lock<std::mutex> lk(srv->mu);
            if (E.active_count() == 0) {
                srv->cv_work.wait(lk, [&] { return !srv->running || !op->queue.empty(); });
                if (!srv->running && op->queue.empty()) return;
            }
            if (!srv->running && op->queue.empty() && E.active_count() == 0) return;
            for (int s = 0; s < op->capacity && !op->queue.empty(); ++s) {
                if (op->slot_busy[s]) continue;
                admit.emplace_back(s, op->queue.front());
                op->queue.pop_front();
                op->slot_busy[s] = true;
            }
        }
        for (auto &a : admit) {
            const int s = a.first;
            std::memcpy(op->pinned_b + (size_t)2 * s * op->n, a.second.b, vb);
            cudaMemcpyAsync(op->stage + (size_t)s * op->n, op->pinned_b + (size_t)2 * s * op->n, vb,
                            cudaMemcpyHostToDevice, op->st);
            E.refine_admit(s, op->stage + (size_t)s * op->n, nullptr, a.second.tol, a.second.max_cycles);
            op->slot_req[s] = a.second;
        }
        std::vector<int> done;
        if (E.refine_cycle(&done) != GDMR_OK) {
            std::lock_guard<std::mutex> lk(srv->mu);
            srv->errors++;
            srv->error = last_error();
            srv->running = false;
            srv->cv_done.notify_all();
            return;
        }
        if (done.empty()) continue;
        for (int s : done)
            cudaMemcpyAsync(op->pinned_x + (size_t)2 * s * op->n, E.slot_x(s), vb, cudaMemcpyDeviceToHost, op->st);
        cudaStreamSynchronize(op->st);
        const auto now = Clock::now();
        std::lock_guard<std::mutex> lk(srv->mu);
        for (int s : done) {
            Request &rq = op->slot_req[s];
            std::memcpy(rq.x, op->pinned_x + (size_t)2 * s * op->n, vb);
            gdmr_stats st{};
            fill_stats(E.slot_stats(s), &st);
            st.latency_ms = std::chrono::duration<double, std::milli>(now - rq.t_submit).count();
            srv->results[rq.ticket] = st;
            srv->finished.push_back(Done{rq.ticket, st});
            op->slot_busy[s] = false;
        }
        srv->cv_done.notify_all();
    }
}

int srv_fail(gdmr_server *srv, int status, const char *what) {
    set_last_error(status, std::string("gdmr_server: ") + what);
    (void)srv;
    return status;
}

}  // namespace

extern "C" long long gdmr_server_slot_bytes(int n, int basisDim, int precision) {
    return (long long)slot_bytes(n, basisDim, precision);
}

// Placement of one operator: the device (index into the budget lists) that keeps the most
// budget free after taking the operator's fixed bytes plus `capacity` slots; capacity <= 0
// asks for as many slots as fit (at most 256) on the device with the most budget free.
// Returns the index, -1 if no device can take the operator with at least one slot.
extern "C" int gdmr_place_operator(int ndev, const long long *budget, const long long *used, long long fixed,
                                   long long per_slot, int capacity, int *capacity_out) {
    int best = -1;
    long long best_left = -1;
    int best_cap = 0;
    for (int d = 0; d < ndev; ++d) {
        const long long room = budget[d] - used[d] - fixed;
        if (room < per_slot) continue;
        const int cap = capacity > 0 ? capacity : (int)std::min(room / per_slot, 256LL);
        const long long left = room - per_slot * cap;
        if (left < 0) continue;
        // with capacity 0 the device with the most room wins (it gets the most slots)
        const long long key = capacity > 0 ? left : room;
        if (key > best_left) {
            best_left = key;
            best = d;
            best_cap = cap;
        }
    }
    if (capacity_out) *capacity_out = best >= 0 ? best_cap : 0;
    return best;
}

extern "C" int gdmr_server_create_multi(gdmr_server **out, long long budget_per_device, const int *devices,
                                        int ndevices) {
    if (!out || budget_per_device <= 0 || !devices || ndevices < 1)
        return srv_fail(nullptr, GDMR_EINVAL, "null output, non-positive budget or empty device list");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) return srv_fail(nullptr, GDMR_ECUDA, "cudaGetDeviceCount");
    for (int i = 0; i < ndevices; ++i)
        if (devices[i] < 0 || devices[i] >= count) return srv_fail(nullptr, GDMR_EINVAL, "device ordinal out of range");
    if (cudaSetDevice(devices[0]) != cudaSuccess) return srv_fail(nullptr, GDMR_ECUDA, "cudaSetDevice");
    auto *s = new gdmr_server();
    s->device = devices[0];
    s->devices.assign(devices, devices + ndevices);
    s->dev_budget.assign(ndevices, budget_per_device);
    s->dev_used.assign(ndevices, 0);
    s->budget = budget_per_device * ndevices;
    *out = s;
    set_last_error(GDMR_OK, "ok");
    return GDMR_OK;
}

extern "C" int gdmr_server_create(gdmr_server **out, long long budget_bytes, int device) {
    return gdmr_server_create_multi(out, budget_bytes, &device, 1);
}

extern "C" int gdmr_server_operator_device(gdmr_server *srv, int op_id) {
    if (!srv || op_id < 0 || op_id >= (int)srv->ops.size()) return -1;
    return srv->ops[op_id]->slot_dev;
}

extern "C" int gdmr_server_add_operator(gdmr_server *srv, int n, const int *rowPtr, const int *colIdx,
                                        const double *vals_ri, int basisDim, int deflatDim, int capacity,
                                        int precision, int *op_id) {
    if (!srv || !op_id) return srv_fail(srv, GDMR_EINVAL, "null argument");
    if (srv->running) return srv_fail(srv, GDMR_EINVAL, "operators are registered before gdmr_server_start");
    if (precision != 0 && precision != 1) return srv_fail(srv, GDMR_EINVAL, "precision must be 0 or 1");
    // the matrix's padded size decides its fixed bytes: count it on the host before placing it
    long padded = 0;
    for (int s0 = 0; s0 < (n + 31) / 32; ++s0) {
        int w = 0;
        for (int r = s0 * 32; r < std::min(n, s0 * 32 + 32); ++r) w = std::max(w, rowPtr[r + 1] - rowPtr[r]);
        padded += 32L * w;
    }
    const long long fixed = (long long)fixed_bytes(n, basisDim, deflatDim, precision, padded);
    const long long per = (long long)slot_bytes(n, basisDim, precision);
    int cap = 0;
    const int slot = gdmr_place_operator((int)srv->devices.size(), srv->dev_budget.data(), srv->dev_used.data(), fixed,
                                         per, capacity, &cap);
    if (slot < 0) return srv_fail(srv, GDMR_ENOMEM, "operator does not fit in the remaining memory budget");
    capacity = cap;
    const int device = srv->devices[slot];
    cudaSetDevice(device);
    std::unique_ptr<ServedOperator> op(new ServedOperator());
    op->id = (int)srv->ops.size();
    op->n = n; op->m = basisDim; op->k = deflatDim; op->precision = precision; op->device = device;
    op->slot_dev = slot;
    if (cudaStreamCreateWithFlags(&op->st, cudaStreamNonBlocking) != cudaSuccess)
        return srv_fail(srv, GDMR_ECUDA, "stream");
    int rc = sell_from_csr(op->A, n, rowPtr, colIdx, vals_ri, precision == 1, true, op->st);
    if (rc != GDMR_OK) return rc;
    op->capacity = capacity;
    if (precision == 1) {
        rc = op->e32.init(n, basisDim, deflatDim, capacity, device);
        op->e32.op.kind = Operator<float>::SELL;
        op->e32.op.sell = op->A.view32();
        op->e32.stream = op->st;
    } else {
        rc = op->e64.init(n, basisDim, deflatDim, capacity, device);
        op->e64.op.kind = Operator<double>::SELL;
        op->e64.op.sell = op->A.view64();
        op->e64.stream = op->st;
    }
    if (rc != GDMR_OK) return rc;
    const size_t vb = sizeof(double2) * (size_t)n * capacity;
    if (cudaMalloc(&op->stage, vb) != cudaSuccess || cudaMallocHost(&op->pinned_b, vb) != cudaSuccess ||
        cudaMallocHost(&op->pinned_x, vb) != cudaSuccess)
        return srv_fail(srv, GDMR_ENOMEM, "staging buffers");
    op->slot_req.resize(capacity);
    op->slot_busy.assign(capacity, false);
    op->bytes = fixed + per * capacity;
    srv->used += op->bytes;
    srv->dev_used[slot] += op->bytes;
    *op_id = op->id;
    srv->ops.push_back(std::move(op));
    set_last_error(GDMR_OK, "ok");
    return GDMR_OK;
}

extern "C" int gdmr_server_operator_capacity(gdmr_server *srv, int op_id) {
    if (!srv || op_id < 0 || op_id >= (int)srv->ops.size()) return 0;
    return srv->ops[op_id]->capacity;
}

extern "C" long long gdmr_server_bytes(gdmr_server *srv) { return srv ? srv->used : 0; }

extern "C" int gdmr_server_start(gdmr_server *srv) {
    if (!srv) return srv_fail(srv, GDMR_EINVAL, "null server");
    if (srv->running) return GDMR_OK;
    srv->running = true;
    for (auto &op : srv->ops) {
        ServedOperator *p = op.get();
        if (p->precision == 1) p->worker = std::thread(worker_loop<float>, srv, p);
        else p->worker = std::thread(worker_loop<double>, srv, p);
    }
    return GDMR_OK;
}

extern "C" int gdmr_server_submit(gdmr_server *srv, int op_id, const double *b, double *x, double tol,
                                  int maxCycles, long long *ticket) {
    if (!srv || !b || !x || !ticket) return srv_fail(srv, GDMR_EINVAL, "null argument");
    if (op_id < 0 || op_id >= (int)srv->ops.size()) return srv_fail(srv, GDMR_EINVAL, "no such operator");
    Request rq;
    rq.ticket = srv->next_ticket++;
    rq.b = b;
    rq.x = x;
    rq.tol = tol;
    rq.max_cycles = maxCycles > 0 ? maxCycles : 5000;
    rq.t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->ops[op_id]->queue.push_back(rq);
    }
    srv->cv_work.notify_all();
    *ticket = rq.ticket;
    return GDMR_OK;
}

extern "C" int gdmr_server_wait(gdmr_server *srv, long long ticket, double timeout_s, gdmr_stats *stats) {
    if (!srv) return srv_fail(srv, GDMR_EINVAL, "null server");
    std::unique_lock<std::mutex> lk(srv->mu);
    const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9);
    while (srv->results.find(ticket) == srv->results.end()) {
        if (srv->errors) return srv_fail(srv, GDMR_ECUDA, srv->error.c_str());
        if (srv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout &&
            srv->results.find(ticket) == srv->results.end())
            return srv_fail(srv, GDMR_ENOCONV, "wait timed out");
    }
    if (stats) *stats = srv->results[ticket];
    srv->results.erase(ticket);
    return GDMR_OK;
}

extern "C" int gdmr_server_poll(gdmr_server *srv, long long *tickets, gdmr_stats *stats, int max) {
    if (!srv) return 0;
    std::lock_guard<std::mutex> lk(srv->mu);
    int c = 0;
    while (c < max && !srv->finished.empty()) {
        Done d = srv->finished.front();
        srv->finished.erase(srv->finished.begin());
        if (tickets) tickets[c] = d.ticket;
        if (stats) stats[c] = d.stats;
        ++c;
    }
    return c;
}

extern "C" int gdmr_server_destroy(gdmr_server *srv) {
    if (!srv) return GDMR_OK;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->running = false;
    }
    srv->cv_work.notify_all();
    for (auto &op : srv->ops)
        if (op->worker.joinable()) op->worker.join();
    srv->ops.clear();   // each operator's destructor frees it on its own device
    delete srv;
    return GDMR_OK;
}
