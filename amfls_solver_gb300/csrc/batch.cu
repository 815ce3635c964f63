// Batched AMFLS: many independent least-squares problems solved
// concurrently on one GPU.  No counterpart in the reference (which solves
// one problem per call); each problem is the reference's solve_amfls.
//
// A pool of host worker threads, each with its own non-blocking CUDA
// stream, takes problems from a shared queue ordered by estimated cost
// (largest first, the LPT rule, so the last problems to start are the
// short ones).  Every solve runs on its worker's stream, so the GPU
// interleaves the levels of up to `workers` problems; small problems, whose
// levels are launch- and latency-bound, share the SMs instead of leaving
// them idle.  A single solve runs each
// checkpoint interval as one CUDA graph (a conditional WHILE node over the
// level), but graphs launched on different streams were measured to run one
// at a time (48 problems, 16 workers: 12.5 s with those graphs, 10.5-12.3 s
// with plain graphs of 2-32 levels, 7.9 s with the level kernels launched
// from the host), so a batch with more than one worker launches from the
// host.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <exception>
#include <numeric>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "batch.hpp"
#include "common.cuh"
#include "csr_operator.hpp"

namespace amfls_gpu {

namespace {

double cost_estimate(const DeviceOperator& op) {
    if (const auto* csr = dynamic_cast<const CsrOperator*>(&op))
        return (double)csr->nonzeros() + op.rows() + op.cols();
    return (double)op.rows() * op.cols();
}

}  // namespace

std::vector<BatchOutcome> solve_amfls_batch(const std::vector<BatchItem>& items, int workers,
                                            double* wall_seconds) {
    const int count = (int)items.size();
    std::vector<BatchOutcome> out(count);
    if (count == 0) {
        if (wall_seconds) *wall_seconds = 0.0;
        return out;
    }
    if (workers <= 0) throw std::invalid_argument("workers must be positive");
    for (const BatchItem& it : items)
        if (it.op == nullptr || it.b == nullptr || it.x == nullptr)
            throw std::invalid_argument("batch problems need an operator, b and a solution buffer");
    {
        // an operator's products use scratch it owns: concurrent solves need one each
        std::vector<const DeviceOperator*> ops;
        for (const BatchItem& it : items) ops.push_back(it.op);
        std::sort(ops.begin(), ops.end());
        if (std::adjacent_find(ops.begin(), ops.end()) != ops.end())
            throw std::invalid_argument("each problem of a batch needs its own operator");
    }
    workers = std::min(workers, count);
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return cost_estimate(*items[a].op) > cost_estimate(*items[b].op);
    });
    int device = 0;
    AMFLS_CUDA(cudaGetDevice(&device));
    std::atomic<int> next{0};
    const auto t0 = std::chrono::steady_clock::now();
    auto work = [&](int w) {
        cudaStream_t s = nullptr;
        try {
            AMFLS_CUDA(cudaSetDevice(device));
            AMFLS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        } catch (...) {
            // the remaining problems are left to the other workers
            return;
        }
        for (int k = next.fetch_add(1); k < count; k = next.fetch_add(1)) {
            const int i = order[k];
            BatchOutcome& o = out[i];
            o.worker = w;
            const auto ts = std::chrono::steady_clock::now();
            try {
                SolveOptions opts = items[i].options;
                // CUDA graphs of different streams were measured to run
                // their work one graph at a time: concurrent solves launch
                // their level kernels from the host instead
                if (workers > 1) opts.use_graphs = false;
                o.result = solve_amfls(*items[i].op, items[i].b, opts, items[i].x, s);
                o.ok = true;
            } catch (const std::exception& e) {
                o.error = e.what();
            } catch (...) {
                o.error = "unknown error";
            }
            o.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - ts).count();
            o.finished = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        cudaStreamDestroy(s);
    };
    std::vector<std::thread> pool;
    pool.reserve(workers);
    for (int w = 0; w < workers; ++w) pool.emplace_back(work, w);
    for (std::thread& t : pool) t.join();
    if (wall_seconds)
        *wall_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    for (int i = 0; i < count; ++i)
        if (!out[i].ok && out[i].error.empty()) out[i].error = "no worker could run the problem";
    return out;
}

}  // namespace amfls_gpu
