// Host-memory helpers of the streamed result path (host code only).
//
// nullh2 = 1 / (1 + delta) is one value per (chromosome, phenotype), repeated over the chromosome's variants in the
// (M, B) table the scan returns (fasterlmm/core.py:717-721).  When results stream to host memory, copying that
// table from the device moves M x B x 8 bytes of repeats over the host link; instead each chromosome's (B,) vector
// is copied and its rows are filled here, on host threads, while the GPU works on the next chromosome.
#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "flmm_common.cuh"

extern "C" int flmm_fill_rows_host_f64(double* dst, int64_t ld, int64_t rows, const double* vec, int64_t n,
                                       int threads) {
    FLMM_REQUIRE(rows >= 0 && n >= 0, "flmm_fill_rows_host_f64: negative size");
    FLMM_REQUIRE(rows == 0 || n == 0 || (dst && vec && ld >= n), "flmm_fill_rows_host_f64: bad arguments");
    if (rows == 0 || n == 0) return FLMM_OK;
    const int64_t want = std::max<int64_t>(1, std::min<int64_t>(threads < 1 ? 1 : threads, 64));
    // at least 256 rows per thread: below that, thread start-up costs more than the copies
    const int64_t nt = std::max<int64_t>(1, std::min<int64_t>(want, rows / 256));
    const size_t bytes = static_cast<size_t>(n) * sizeof(double);
    auto fill = [=](int64_t r0, int64_t r1) {
        for (int64_t r = r0; r < r1; ++r) std::memcpy(dst + r * ld, vec, bytes);
    };
    if (nt == 1) {
        fill(0, rows);
        return FLMM_OK;
    }
    std::vector<std::thread> pool;
    pool.reserve(static_cast<size_t>(nt));
    for (int64_t t = 0; t < nt; ++t) pool.emplace_back(fill, rows * t / nt, rows * (t + 1) / nt);
    for (auto& th : pool) th.join();
    return FLMM_OK;
}

extern "C" int flmm_host_alloc_mapped(size_t bytes, void** host_ptr, void** dev_ptr) {
    FLMM_REQUIRE(host_ptr && dev_ptr && bytes > 0, "flmm_host_alloc_mapped: bad arguments");
    *host_ptr = nullptr;
    *dev_ptr = nullptr;
    void* h = nullptr;
    FLMM_CUDA(cudaHostAlloc(&h, bytes, cudaHostAllocMapped));
    void* d = nullptr;
    const cudaError_t e = cudaHostGetDevicePointer(&d, h, 0);
    if (e != cudaSuccess || d == nullptr) {
        cudaFreeHost(h);
        return flmm::fail(FLMM_ERR_CUDA, "flmm_host_alloc_mapped: no device mapping (%s)", cudaGetErrorString(e));
    }
    *host_ptr = h;
    *dev_ptr = d;
    return FLMM_OK;
}

extern "C" int flmm_host_free_mapped(void* host_ptr) {
    if (host_ptr) FLMM_CUDA(cudaFreeHost(host_ptr));
    return FLMM_OK;
}
