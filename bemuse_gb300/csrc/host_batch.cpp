// host_batch.cpp -- many independent bodies at once.  Each body is the
// reference's per-body loop (Setup, then Set_Real + Solve per frequency;
// BEMUser_Console.cpp:242-262); bodies are independent, so a pool of host
// threads, each driving its own context (its own streams and buffers on the
// same GPU), runs several body pipelines concurrently.  Bodies are taken
// largest first from a shared counter, which balances uneven panel counts.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bemgpu.h"
#include "bem_internal.h"

extern "C" bem_status bem_batch_solve(int device, int n_bodies, const bem_mesh* meshes, const bem_body_props* props,
                                      double density, double gravity, int n_beta, const double* betas, int n_freq,
                                      const double* omega, int precision, double tol, int n_workers,
                                      bem_result* results, double* seconds) {
    if (n_bodies < 0 || (n_bodies > 0 && (!meshes || !results)) || n_freq < 0 || (n_freq > 0 && !omega) ||
        n_beta < 0 || (n_beta > 0 && !betas)) {
        bem::set_static_error("bem_batch_solve: bad arguments");
        return BEM_ERR_ARG;
    }
    if (n_workers <= 0) n_workers = 8;
    n_workers = std::max(1, std::min(n_workers, std::max(1, n_bodies)));
    std::vector<int> order(n_bodies);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return meshes[a].n_elems > meshes[b].n_elems; });
    std::atomic<int> next{0};
    std::mutex mu;
    bem_status first = BEM_OK;
    std::string first_msg;
    auto record = [&](bem_status s, const std::string& msg) {
        std::lock_guard<std::mutex> g(mu);
        if (first == BEM_OK) {
            first = s;
            first_msg = msg;
        }
    };
    const auto t0 = std::chrono::steady_clock::now();
    auto worker = [&]() {
        bem_ctx* ctx = nullptr;
        bem_status s = bem_create(&ctx, device);
        if (s != BEM_OK) {
            record(s, bem_last_error(nullptr));
            return;
        }
        s = bem_set_params(ctx, density, gravity, n_beta, betas);
        if (s != BEM_OK) record(s, bem_last_error(ctx));
        // The default share of SMs kept free of a context's assembly suits one pipeline
        // on the GPU; with several, the other contexts' work fills those SMs anyway, and
        // a smaller reserve measured faster (24 SMs).
        if (s == BEM_OK && n_workers > 1) {
            s = bem_set_tuning(ctx, "asm_reserve_sms", 24);
            if (s != BEM_OK) record(s, bem_last_error(ctx));
        }
        while (s == BEM_OK) {
            const int k = next.fetch_add(1);
            if (k >= n_bodies) break;
            const int b = order[k];
            bem_body_props p = {};
            if (props) p = props[b];
            s = bem_setup(ctx, &meshes[b], &p);
            if (s == BEM_OK) s = bem_solve(ctx, n_freq, omega, precision, tol, &results[b]);
            if (s != BEM_OK) {
                record(s, std::string("body ") + std::to_string(b) + ": " + bem_last_error(ctx));
                break;
            }
        }
        bem_destroy(ctx);
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < n_workers; ++w) pool.emplace_back(worker);
    for (auto& t : pool) t.join();
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (first != BEM_OK) bem::set_static_error(("bem_batch_solve: " + first_msg).c_str());
    return first;
}
