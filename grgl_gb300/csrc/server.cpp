// The serving loop behind grgx_server_*: resident graphs, a request queue, and worker threads
// that coalesce compatible queued requests into one traversal each (continuous batching).
//
// Each worker owns a CUDA stream.  A free worker takes the oldest queued request and every other
// queued request for the same graph, direction and dtype whose rows still fit the batch width,
// reserves the batch's estimated device memory against the budget (waiting while other batches
// hold it), runs the batch through matmul_batch_impl on its stream and completes the tickets.
// Workers run concurrently, so batches overlap on the device; requests arriving meanwhile are
// picked up by whichever worker frees first.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "grgx_internal.h"

namespace grgx {

void matmul_batch_impl(grgx_graph* g, const grgx_request* reqs, uint64_t n, uint64_t maxCols, uint32_t flags,
                       void* stream);
uint64_t default_batch_cols(int dtype);
struct DevicePlan;
DevicePlan* ensure_device_plan(grgx_graph* g);

}  // namespace grgx

struct grgx_server {
    struct Req {
        uint64_t ticket = 0;
        uint32_t graph = 0;
        grgx_request r{};
        double submit = 0, start = 0, done = 0;
        uint64_t batchReqs = 0, batchRows = 0;
        bool finished = false;
        int status = GRGX_OK;
        std::string err;
    };
    int device = 0;
    uint64_t budget = 0, reserved = 0, maxCols = 0;
    uint32_t inFlight = 0;
    std::vector<grgx_graph*> graphs;
    std::deque<std::shared_ptr<Req>> pending;
    std::map<uint64_t, std::shared_ptr<Req>> tickets;
    uint64_t nextTicket = 1;
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::vector<std::thread> workers;
    bool stop = false;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }

    static size_t elem(int dtype) {
        switch (dtype) {
        case GRGX_F64: case GRGX_I64: case GRGX_U64: return 8;
        case GRGX_F32: case GRGX_I32: case GRGX_U32: return 4;
        case GRGX_I16: case GRGX_U16: return 2;
        default: return 1;
        }
    }

    // Conservative device bytes of one batch: node values and per-mutation rows in the widest
    // storage (8 bytes), the stacked input/output, plus a quarter for partials and the pool.
    uint64_t estimate(const grgx::HostGraph& h, int dtype, uint64_t rows) const {
        const uint64_t es = elem(dtype);
        // node values and the DOWN input rows (8 bytes an element at most), the split-form UP
        // state (16 bytes an element at most), heavy-row partials (a quarter more), and the I/O
        const uint64_t valueBytes = (h.num_nodes + h.num_mutations) * rows * 8;
        const uint64_t stateBytes = h.num_nodes * rows * 16;
        const uint64_t ioBytes = rows * (h.num_samples + h.num_mutations) * es * 2;
        return valueBytes + valueBytes / 4 + stateBytes + ioBytes;
    }

    void worker_main() {
        cudaSetDevice(device);
        cudaStream_t stream = nullptr;
        cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
        for (;;) {
            std::vector<std::shared_ptr<Req>> batch;
            uint64_t rows = 0, bytes = 0;
            {
                std::unique_lock<std::mutex> lk(mu);
                for (;;) {
                    if (stop) {
                        if (stream) cudaStreamDestroy(stream);
                        return;
                    }
                    if (pending.empty()) {
                        cvWork.wait(lk);
                        continue;
                    }
                    // form the batch: the oldest request and compatible followers
                    const std::shared_ptr<Req> head = pending.front();
                    const grgx::HostGraph& h = *graphs[head->graph]->host;
                    const uint64_t width = maxCols ? maxCols : grgx::default_batch_cols(head->r.dtype);
                    std::vector<size_t> take{0};
                    rows = head->r.rows;
                    for (size_t i = 1; i < pending.size(); i++) {
                        const Req& q = *pending[i];
                        const bool sameFold = ((q.r.options ^ head->r.options) & GRGX_REQUEST_BY_INDIVIDUAL) == 0;
                        if (q.graph == head->graph && q.r.direction == head->r.direction && q.r.dtype == head->r.dtype &&
                            sameFold && rows + q.r.rows <= width) {
                            take.push_back(i);
                            rows += q.r.rows;
                        }
                    }
                    bytes = estimate(h, head->r.dtype, rows);
                    if (bytes > budget && inFlight == 0 && take.size() == 1) {
                        // can never fit: fail it rather than wait forever
                        head->finished = true;
                        head->status = GRGX_ERR_OUT_OF_MEMORY;
                        head->err = "request needs about " + std::to_string(bytes) +
                                    " device bytes, more than the server's memory budget of " + std::to_string(budget);
                        head->done = now();
                        pending.pop_front();
                        cvDone.notify_all();
                        continue;
                    }
                    if (reserved + bytes > budget) {
                        if (inFlight == 0 && take.size() > 1) {
                            // shrink to the head request alone
                            take.resize(1);
                            rows = head->r.rows;
                            bytes = estimate(h, head->r.dtype, rows);
                            if (reserved + bytes > budget) {
                                cvWork.wait(lk);
                                continue;
                            }
                        } else {
                            cvWork.wait(lk);  // admission: wait for memory held by batches in flight
                            continue;
                        }
                    }
                    const double t = now();
                    for (size_t k = take.size(); k > 0; k--) {
                        batch.push_back(pending[take[k - 1]]);
                        pending.erase(pending.begin() + static_cast<long>(take[k - 1]));
                    }
                    std::reverse(batch.begin(), batch.end());
                    for (auto& q : batch) {
                        q->start = t;
                        q->batchReqs = batch.size();
                        q->batchRows = rows;
                    }
                    reserved += bytes;
                    inFlight++;
                    break;
                }
            }
            // run the batch on this worker's stream
            std::vector<grgx_request> reqs;
            for (auto& q : batch) reqs.push_back(q->r);
            int status = GRGX_OK;
            std::string err;
            try {
                grgx::matmul_batch_impl(graphs[batch[0]->graph], reqs.data(), reqs.size(), rows, GRGX_FLAG_SYNC,
                                        stream);
            } catch (const grgx::Error& e) {
                status = e.code;
                err = e.what();
            } catch (const std::exception& e) {
                status = GRGX_ERR_CUDA;
                err = e.what();
            }
            {
                std::lock_guard<std::mutex> lk(mu);
                const double t = now();
                for (auto& q : batch) {
                    q->finished = true;
                    q->status = status;
                    q->err = err;
                    q->done = t;
                }
                reserved -= bytes;
                inFlight--;
            }
            cvDone.notify_all();
            cvWork.notify_all();
        }
    }
};

using grgx::Error;

namespace grgx {
namespace {
template <typename F> grgx_status server_guard(F&& f) {
    try {
        f();
        set_last_error("");
        return GRGX_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return static_cast<grgx_status>(e.code);
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return GRGX_ERR_CUDA;
    }
}
}  // namespace
}  // namespace grgx

extern "C" {

grgx_status grgx_server_create(uint32_t workers, uint64_t memory_budget, uint64_t max_cols, grgx_server** out) {
    return grgx::server_guard([&] {
        GRGX_CHECK(out != nullptr && workers > 0 && workers <= 64, GRGX_ERR_API_MISUSE, "workers must be in 1..64");
        auto s = std::make_unique<grgx_server>();
        GRGX_CHECK(cudaGetDevice(&s->device) == cudaSuccess, GRGX_ERR_NO_DEVICE, "no CUDA device");
        size_t freeB = 0, totalB = 0;
        GRGX_CHECK(cudaMemGetInfo(&freeB, &totalB) == cudaSuccess, GRGX_ERR_NO_DEVICE, "cudaMemGetInfo failed");
        s->budget = memory_budget ? memory_budget : static_cast<uint64_t>(freeB * 0.9);
        s->maxCols = max_cols;
        grgx_server* raw = s.get();
        for (uint32_t i = 0; i < workers; i++) s->workers.emplace_back([raw] { raw->worker_main(); });
        *out = s.release();
    });
}

grgx_status grgx_server_add_graph(grgx_server* s, grgx_graph* g, uint32_t* graph_id) {
    return grgx::server_guard([&] {
        GRGX_CHECK(s && g && graph_id, GRGX_ERR_API_MISUSE, "null argument");
        int dev = 0;
        cudaGetDevice(&dev);
        cudaSetDevice(s->device);
        grgx::ensure_device_plan(g);
        cudaSetDevice(dev);
        std::lock_guard<std::mutex> lk(s->mu);
        s->graphs.push_back(g);
        *graph_id = static_cast<uint32_t>(s->graphs.size() - 1);
    });
}

grgx_status grgx_server_submit(grgx_server* s, uint32_t graph_id, const grgx_request* request, uint64_t* ticket) {
    return grgx::server_guard([&] {
        GRGX_CHECK(s && request && ticket, GRGX_ERR_API_MISUSE, "null argument");
        GRGX_CHECK(request->input && request->output && request->rows > 0, GRGX_ERR_API_MISUSE,
                   "matmul() requires non-zero dimensions.");
        GRGX_CHECK(request->direction == GRGX_DIRECTION_DOWN || request->direction == GRGX_DIRECTION_UP,
                   GRGX_ERR_API_MISUSE, "Invalid traversal direction");
        GRGX_CHECK(request->dtype >= GRGX_F64 && request->dtype <= GRGX_BOOL, GRGX_ERR_API_MISUSE,
                   "Unsupported dtype");
        GRGX_CHECK((request->options & ~(GRGX_REQUEST_STANDARDIZED | GRGX_REQUEST_BY_INDIVIDUAL)) == 0,
                   GRGX_ERR_API_MISUSE,
                   "Unknown request options");
        GRGX_CHECK(!(request->options & GRGX_REQUEST_STANDARDIZED) || request->dtype == GRGX_F32 ||
                       request->dtype == GRGX_F64,
                   GRGX_ERR_UNSUPPORTED, "standardized products take float32 or float64 input");
        auto q = std::make_shared<grgx_server::Req>();
        q->r = *request;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            GRGX_CHECK(graph_id < s->graphs.size(), GRGX_ERR_API_MISUSE, "unknown graph id");
            GRGX_CHECK(!s->stop, GRGX_ERR_API_MISUSE, "server is stopping");
            q->graph = graph_id;
            q->ticket = s->nextTicket++;
            q->submit = s->now();
            s->tickets[q->ticket] = q;
            s->pending.push_back(q);
            *ticket = q->ticket;
        }
        s->cvWork.notify_one();
    });
}

grgx_status grgx_server_wait(grgx_server* s, uint64_t ticket, double timeout_s, grgx_request_stats* stats) {
    std::shared_ptr<grgx_server::Req> q;
    grgx_status st = grgx::server_guard([&] {
        GRGX_CHECK(s != nullptr, GRGX_ERR_API_MISUSE, "null argument");
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->tickets.find(ticket);
        GRGX_CHECK(it != s->tickets.end(), GRGX_ERR_API_MISUSE, "unknown ticket");
        q = it->second;
        const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
        while (!q->finished) {
            if (timeout_s > 0) {
                if (s->cvDone.wait_until(lk, deadline) == std::cv_status::timeout && !q->finished)
                    throw Error(GRGX_ERR_TIMEOUT, "timed out waiting for the request");
            } else {
                s->cvDone.wait(lk);
            }
        }
        s->tickets.erase(ticket);
    });
    if (st != GRGX_OK) return st;
    if (stats) {
        stats->submit_s = q->submit;
        stats->start_s = q->start;
        stats->done_s = q->done;
        stats->batch_requests = q->batchReqs;
        stats->batch_rows = q->batchRows;
    }
    grgx::set_last_error(q->err);
    return static_cast<grgx_status>(q->status);
}

void grgx_server_destroy(grgx_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (auto& q : s->pending) {
            q->finished = true;
            q->status = GRGX_ERR_TIMEOUT;
            q->err = "server stopped before the request ran";
        }
        s->pending.clear();
    }
    s->cvWork.notify_all();
    s->cvDone.notify_all();
    for (auto& t : s->workers) t.join();
    delete s;
}

}  // extern "C"
