// Library-level entry points: status strings, per-thread last error, the per-device context (cuSOLVER handle),
// and the two FP64 factorisations that go through cuSOLVER: the covariate SVD (the pseudo-inverse of
// fasterlmm/core.py:498) and the kinship eigendecomposition (fasterlmm/core.py:54-77, :510).
#include <cusolverDn.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include <mutex>

#include "flmm_common.cuh"

constexpr int kEighWorkers = 8;
constexpr int kFlagSlots = 64;

struct flmm_context {
    int device = 0;
    int sm_count = 0;
    cusolverDnHandle_t solver = nullptr;
    int* err_flag = nullptr;  // device int raised by kernels whose bounded waits time out
    // mapped host copies of the flags for flmm_context_check (kFlagSlots pairs, one per concurrent call): a kernel
    // writes them over the host link, so reading them never queues on the copy engines behind a scan's streamed
    // result copies
    int* flags_host = nullptr;
    int* flags_dev = nullptr;
    std::atomic<unsigned> flag_slot{0};
    // worker streams / handles for running independent eigendecompositions side by side
    cudaStream_t workers[kEighWorkers] = {};
    cusolverDnHandle_t wsolver[kEighWorkers] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kEighWorkers] = {};
    cusolverDnParams_t params = nullptr;
};

namespace flmm {

static thread_local char g_last_error[512] = {0};

int fail(int status, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return status;
}

static std::atomic<unsigned long long> g_launches{0};

int check_cuda(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(FLMM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return FLMM_OK;
}

int check_launch(const char* what) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return check_cuda(what);
}

static int solver_fail(cusolverStatus_t st, const char* what) {
    return fail(FLMM_ERR_SOLVER, "%s: cusolver status %d", what, static_cast<int>(st));
}

}  // namespace flmm

using namespace flmm;

extern "C" int flmm_version(void) { return 100; }

extern "C" const char* flmm_status_string(int status) {
    switch (status) {
        case FLMM_OK: return "ok";
        case FLMM_ERR_ARG: return "invalid argument";
        case FLMM_ERR_CUDA: return "CUDA error";
        case FLMM_ERR_SOLVER: return "cuSOLVER error";
        case FLMM_ERR_WORKSPACE: return "workspace too small";
        case FLMM_ERR_DEVICE: return "unsupported device (needs sm_103, GB300)";
        case FLMM_ERR_TIMEOUT: return "bounded device wait timed out";
        default: return "unknown status";
    }
}

extern "C" const char* flmm_last_error(void) { return g_last_error; }

extern "C" uint64_t flmm_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" int flmm_context_destroy(flmm_context* ctx);

extern "C" int flmm_context_create(int device, flmm_context** out) {
    FLMM_REQUIRE(out != nullptr, "flmm_context_create: out is NULL");
    *out = nullptr;
    cudaDeviceProp prop;
    FLMM_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major != 10 || prop.minor != 3)
        return fail(FLMM_ERR_DEVICE, "device %d is sm_%d%d (%s); the library is compiled for sm_103a only", device, prop.major,
                    prop.minor, prop.name);
    FLMM_CUDA(cudaSetDevice(device));
    flmm_context* ctx = new (std::nothrow) flmm_context();
    if (!ctx) return fail(FLMM_ERR_ARG, "flmm_context_create: out of host memory");
    ctx->device = device;
    ctx->sm_count = prop.multiProcessorCount;
    cusolverStatus_t st = cusolverDnCreate(&ctx->solver);
    if (st != CUSOLVER_STATUS_SUCCESS) {
        delete ctx;
        return solver_fail(st, "cusolverDnCreate");
    }
    if (cudaMalloc(&ctx->err_flag, sizeof(int)) != cudaSuccess || cudaMemset(ctx->err_flag, 0, sizeof(int)) != cudaSuccess) {
        cusolverDnDestroy(ctx->solver);
        delete ctx;
        return fail(FLMM_ERR_CUDA, "flmm_context_create: cannot allocate the device error flag");
    }
    if (cudaHostAlloc(&ctx->flags_host, 2 * kFlagSlots * sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(&ctx->flags_dev, ctx->flags_host, 0) != cudaSuccess) {
        flmm_context_destroy(ctx);
        return fail(FLMM_ERR_CUDA, "flmm_context_create: cannot allocate the mapped flag buffer");
    }
    bool ok = cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming) == cudaSuccess &&
              cusolverDnCreateParams(&ctx->params) == CUSOLVER_STATUS_SUCCESS;
    for (int w = 0; ok && w < kEighWorkers; ++w) {
        ok = cudaStreamCreateWithFlags(&ctx->workers[w], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&ctx->join[w], cudaEventDisableTiming) == cudaSuccess &&
             cusolverDnCreate(&ctx->wsolver[w]) == CUSOLVER_STATUS_SUCCESS &&
             cusolverDnSetStream(ctx->wsolver[w], ctx->workers[w]) == CUSOLVER_STATUS_SUCCESS;
    }
    if (!ok) {
        flmm_context_destroy(ctx);
        return fail(FLMM_ERR_CUDA, "flmm_context_create: cannot create worker streams / solver handles");
    }
    *out = ctx;
    return FLMM_OK;
}

int flmm_ctx_sm_count(flmm_context* ctx) { return ctx->sm_count; }
int* flmm_ctx_err_flag(flmm_context* ctx) { return ctx->err_flag; }

int* flmm::device_err_flag(int device) {
    static std::mutex mu;
    static int* flags[64] = {};
    if (device < 0 || device >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!flags[device]) {
        int prev = 0;
        if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) return nullptr;
        int* f = nullptr;
        if (cudaMalloc(&f, sizeof(int)) == cudaSuccess && cudaMemset(f, 0, sizeof(int)) == cudaSuccess) flags[device] = f;
        cudaSetDevice(prev);
    }
    return flags[device];
}

// both error flags into the context's mapped host buffer
__global__ void k_read_flags(const int* __restrict__ ctx_flag, const int* __restrict__ dev_flag, int* out) {
    if (threadIdx.x == 0) {
        out[0] = *reinterpret_cast<const volatile int*>(ctx_flag);
        out[1] = dev_flag ? *reinterpret_cast<const volatile int*>(dev_flag) : 0;
    }
}

extern "C" int flmm_context_check(flmm_context* ctx, void* stream) {
    FLMM_REQUIRE(ctx, "flmm_context_check: NULL context");
    int* dflag = device_err_flag(ctx->device);
    const unsigned slot = ctx->flag_slot.fetch_add(1u) % kFlagSlots;
    volatile int* hf = ctx->flags_host + 2 * slot;
    hf[0] = 0;
    hf[1] = 0;
    k_read_flags<<<1, 32, 0, as_stream(stream)>>>(ctx->err_flag, dflag, ctx->flags_dev + 2 * slot);
    int rc = check_launch("k_read_flags");
    if (rc) return rc;
    FLMM_CUDA(cudaStreamSynchronize(as_stream(stream)));
    const int h[2] = {hf[0], hf[1]};
    if (h[0] != 0 || h[1] != 0) {
        FLMM_CUDA(cudaMemsetAsync(ctx->err_flag, 0, sizeof(int), as_stream(stream)));
        if (dflag) FLMM_CUDA(cudaMemsetAsync(dflag, 0, sizeof(int), as_stream(stream)));
        return fail(FLMM_ERR_TIMEOUT, "a tensor-core kernel gave up a bounded wait (code %d)", h[0] ? h[0] : h[1]);
    }
    return FLMM_OK;
}

extern "C" int flmm_context_destroy(flmm_context* ctx) {
    if (!ctx) return FLMM_OK;
    if (ctx->solver) cusolverDnDestroy(ctx->solver);
    if (ctx->err_flag) cudaFree(ctx->err_flag);
    if (ctx->flags_host) cudaFreeHost(ctx->flags_host);
    for (int w = 0; w < kEighWorkers; ++w) {
        if (ctx->wsolver[w]) cusolverDnDestroy(ctx->wsolver[w]);
        if (ctx->workers[w]) cudaStreamDestroy(ctx->workers[w]);
        if (ctx->join[w]) cudaEventDestroy(ctx->join[w]);
    }
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    if (ctx->params) cusolverDnDestroyParams(ctx->params);
    delete ctx;
    return FLMM_OK;
}

// ---- eigendecomposition -------------------------------------------------------------------------------------

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

extern "C" int flmm_eigh_workspace_bytes(flmm_context* ctx, int N, size_t* bytes) {
    FLMM_REQUIRE(ctx && bytes && N > 0, "flmm_eigh_workspace_bytes: bad arguments");
    int lwork = 0;
    cusolverStatus_t st = cusolverDnDsyevd_bufferSize(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER,
                                                      N, nullptr, N, nullptr, &lwork);
    if (st != CUSOLVER_STATUS_SUCCESS) return solver_fail(st, "cusolverDnDsyevd_bufferSize");
    *bytes = align_up(sizeof(double) * static_cast<size_t>(lwork), 256) + 256;
    return FLMM_OK;
}

extern "C" int flmm_eigh(flmm_context* ctx, double* A, int N, double* evals, void* work, size_t work_bytes,
                         void* stream) {
    FLMM_REQUIRE(ctx && A && evals && work && N > 0, "flmm_eigh: bad arguments");
    size_t need = 0;
    int rc = flmm_eigh_workspace_bytes(ctx, N, &need);
    if (rc) return rc;
    if (work_bytes < need) return fail(FLMM_ERR_WORKSPACE, "flmm_eigh: need %zu bytes, got %zu", need, work_bytes);
    int lwork = static_cast<int>((need - 256) / sizeof(double));
    double* dwork = static_cast<double*>(work);
    int* info = reinterpret_cast<int*>(static_cast<char*>(work) + need - 256);
    cusolverDnSetStream(ctx->solver, as_stream(stream));
    // symmetric input: row-major and column-major views coincide; the eigenvector k comes back as column k of the
    // column-major result, i.e. row k of the row-major view
    cusolverStatus_t st = cusolverDnDsyevd(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, N, A, N,
                                           evals, dwork, lwork, info);
    if (st != CUSOLVER_STATUS_SUCCESS) return solver_fail(st, "cusolverDnDsyevd");
    return check_cuda("cusolverDnDsyevd");
}

// ---- batched eigendecomposition: all LOCO kinships of a scan at once --------------------------------------------

namespace {

struct BatchedLayout {
    size_t dev_bytes, host_bytes;
};

int batched_api_sizes(flmm_context* ctx, int N, int batch, BatchedLayout* L) {
    size_t dbytes = 0, hbytes = 0;
    cusolverStatus_t st = cusolverDnXsyevBatched_bufferSize(ctx->solver, ctx->params, CUSOLVER_EIG_MODE_VECTOR,
                                                            CUBLAS_FILL_MODE_LOWER, N, CUDA_R_64F, nullptr, N,
                                                            CUDA_R_64F, nullptr, CUDA_R_64F, &dbytes, &hbytes, batch);
    if (st != CUSOLVER_STATUS_SUCCESS) return solver_fail(st, "cusolverDnXsyevBatched_bufferSize");
    L->dev_bytes = align_up(dbytes, 256) + align_up(sizeof(int) * batch, 256);
    L->host_bytes = hbytes;
    return FLMM_OK;
}

}  // namespace

extern "C" int flmm_eigh_batched_workspace_bytes(flmm_context* ctx, int N, int batch, int mode, size_t* bytes) {
    FLMM_REQUIRE(ctx && bytes && N > 0 && batch > 0 && (mode == 1 || mode == 2),
                 "flmm_eigh_batched_workspace_bytes: bad arguments (mode 1 = batched API, 2 = concurrent syevd)");
    if (mode == 1) {
        BatchedLayout L;
        int rc = batched_api_sizes(ctx, N, batch, &L);
        if (rc) return rc;
        if (L.host_bytes != 0)
            return fail(FLMM_ERR_SOLVER, "cusolverDnXsyevBatched needs %zu bytes of host workspace", L.host_bytes);
        *bytes = L.dev_bytes;
        return FLMM_OK;
    }
    size_t one = 0;
    int rc = flmm_eigh_workspace_bytes(ctx, N, &one);
    if (rc) return rc;
    const int slots = batch < kEighWorkers ? batch : kEighWorkers;
    *bytes = one * static_cast<size_t>(slots);
    return FLMM_OK;
}

extern "C" int flmm_eigh_batched(flmm_context* ctx, double* A, int N, int batch, double* evals, int mode, int slot,
                                 void* work, size_t work_bytes, void* stream) {
    FLMM_REQUIRE(ctx && A && evals && work && N > 0 && batch > 0 && slot >= -1 && slot < kEighWorkers,
                 "flmm_eigh_batched: bad arguments");
    size_t need = 0;
    int rc = flmm_eigh_batched_workspace_bytes(ctx, N, batch, mode, &need);
    if (rc) return rc;
    if (work_bytes < need)
        return fail(FLMM_ERR_WORKSPACE, "flmm_eigh_batched: need %zu bytes, got %zu", need, work_bytes);
    cudaStream_t st = as_stream(stream);
    const size_t nn = static_cast<size_t>(N) * N;
    if (mode == 1) {
        BatchedLayout L;
        if ((rc = batched_api_sizes(ctx, N, batch, &L))) return rc;
        int* info = reinterpret_cast<int*>(static_cast<char*>(work) + (L.dev_bytes - align_up(sizeof(int) * batch, 256)));
        cusolverDnHandle_t hdl = slot < 0 ? ctx->solver : ctx->wsolver[slot];
        cusolverDnSetStream(hdl, st);
        cusolverStatus_t cs = cusolverDnXsyevBatched(hdl, ctx->params, CUSOLVER_EIG_MODE_VECTOR,
                                                     CUBLAS_FILL_MODE_LOWER, N, CUDA_R_64F, A, N, CUDA_R_64F, evals,
                                                     CUDA_R_64F, work, L.dev_bytes, nullptr, 0, info, batch);
        if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail(cs, "cusolverDnXsyevBatched");
        return check_cuda("cusolverDnXsyevBatched");
    }
    // mode 2: independent syevd calls spread over the worker streams, forked from and joined back into `stream`
    size_t one = 0;
    if ((rc = flmm_eigh_workspace_bytes(ctx, N, &one))) return rc;
    const int slots = batch < kEighWorkers ? batch : kEighWorkers;
    const int lwork = static_cast<int>((one - 256) / sizeof(double));
    FLMM_CUDA(cudaEventRecord(ctx->fork, st));
    for (int w = 0; w < slots; ++w) FLMM_CUDA(cudaStreamWaitEvent(ctx->workers[w], ctx->fork, 0));
    for (int w = 0; w < slots; ++w) cusolverDnSetStream(ctx->wsolver[w], ctx->workers[w]);
    for (int b = 0; b < batch; ++b) {
        const int w = b % slots;
        char* wbase = static_cast<char*>(work) + one * static_cast<size_t>(w);
        int* info = reinterpret_cast<int*>(wbase + one - 256);
        cusolverStatus_t cs = cusolverDnDsyevd(ctx->wsolver[w], CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, N,
                                               A + nn * b, N, evals + static_cast<size_t>(N) * b,
                                               reinterpret_cast<double*>(wbase), lwork, info);
        if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail(cs, "cusolverDnDsyevd (worker)");
    }
    for (int w = 0; w < slots; ++w) {
        FLMM_CUDA(cudaEventRecord(ctx->join[w], ctx->workers[w]));
        FLMM_CUDA(cudaStreamWaitEvent(st, ctx->join[w], 0));
    }
    return check_cuda("flmm_eigh_batched");
}

// ---- single-precision batched eigendecomposition (fast form) -----------------------------------------------------
//
// The fast form carries the eigenbasis as split-FP16 operands (~2^-22 relative) and its spectrum in FP32, so an FP32
// eigendecomposition (backward error ~1e-7 of the projected kinship) is below the precision it is used at.

namespace {

// Small batches from this N on go one matrix at a time through cusolverDnSsyevd: measured on GB300 per matrix, the
// batched call on 4 matrices takes 65 ms at N = 3,000 (syevd 46) and on 2 at N = 5,000 281 ms (109); on 22 matrices
// of N = 3,000-5,000 the batched call is the faster one (49.9 s against 57.5 s for 12 such batches).
constexpr int kSyevdFromN = 2500;
constexpr int kSyevdMaxBatch = 4;

int syevd_f32_lwork(flmm_context* ctx, int N, int* lwork) {
    cusolverStatus_t st = cusolverDnSsyevd_bufferSize(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, N,
                                                      nullptr, N, nullptr, lwork);
    if (st != CUSOLVER_STATUS_SUCCESS) return solver_fail(st, "cusolverDnSsyevd_bufferSize");
    return FLMM_OK;
}

// Below kSyevdFromN the library's own batched solver (csrc/flmm_eigh_own.cu) runs unless FLMM_EIGH_F32=cusolver
// selects cuSOLVER's batched call.
bool own_solver(int N) {
    if (N >= kSyevdFromN) return false;
    static const bool cus = [] {
        const char* v = getenv("FLMM_EIGH_F32");
        return v != nullptr && strcmp(v, "cusolver") == 0;
    }();
    return !cus;
}

bool syevd_loop(int N, int batch) { return N >= kSyevdFromN && batch <= kSyevdMaxBatch; }

int batched_api_sizes_f32(flmm_context* ctx, int N, int batch, BatchedLayout* L) {
    if (own_solver(N)) {
        L->dev_bytes = eigh_own_workspace_bytes(N, batch);
        L->host_bytes = 0;
        return FLMM_OK;
    }
    if (syevd_loop(N, batch)) {
        int lwork = 0;
        int rc = syevd_f32_lwork(ctx, N, &lwork);
        if (rc) return rc;
        L->dev_bytes = align_up(sizeof(float) * static_cast<size_t>(lwork), 256) + align_up(sizeof(int) * batch, 256);
        L->host_bytes = 0;
        return FLMM_OK;
    }
    size_t dbytes = 0, hbytes = 0;
    cusolverStatus_t st = cusolverDnXsyevBatched_bufferSize(ctx->solver, ctx->params, CUSOLVER_EIG_MODE_VECTOR,
                                                            CUBLAS_FILL_MODE_LOWER, N, CUDA_R_32F, nullptr, N,
                                                            CUDA_R_32F, nullptr, CUDA_R_32F, &dbytes, &hbytes, batch);
    if (st != CUSOLVER_STATUS_SUCCESS) return solver_fail(st, "cusolverDnXsyevBatched_bufferSize (FP32)");
    L->dev_bytes = align_up(dbytes, 256) + align_up(sizeof(int) * batch, 256);
    L->host_bytes = hbytes;
    return FLMM_OK;
}

}  // namespace

extern "C" int flmm_eigh_batched_f32_workspace_bytes(flmm_context* ctx, int N, int batch, size_t* bytes) {
    FLMM_REQUIRE(ctx && bytes && N > 0 && batch > 0, "flmm_eigh_batched_f32_workspace_bytes: bad arguments");
    BatchedLayout L;
    int rc = batched_api_sizes_f32(ctx, N, batch, &L);
    if (rc) return rc;
    if (L.host_bytes != 0)
        return fail(FLMM_ERR_SOLVER, "cusolverDnXsyevBatched (FP32) needs %zu bytes of host workspace", L.host_bytes);
    *bytes = L.dev_bytes;
    return FLMM_OK;
}

extern "C" int flmm_eigh_batched_f32(flmm_context* ctx, float* A, int N, int batch, float* evals, void* work,
                                     size_t work_bytes, void* stream) {
    FLMM_REQUIRE(ctx && A && evals && work && N > 0 && batch > 0, "flmm_eigh_batched_f32: bad arguments");
    size_t need = 0;
    int rc = flmm_eigh_batched_f32_workspace_bytes(ctx, N, batch, &need);
    if (rc) return rc;
    if (work_bytes < need)
        return fail(FLMM_ERR_WORKSPACE, "flmm_eigh_batched_f32: need %zu bytes, got %zu", need, work_bytes);
    BatchedLayout L;
    if ((rc = batched_api_sizes_f32(ctx, N, batch, &L))) return rc;
    if (own_solver(N)) return eigh_own_f32(A, N, batch, evals, work, as_stream(stream));
    int* info = reinterpret_cast<int*>(static_cast<char*>(work) + (L.dev_bytes - align_up(sizeof(int) * batch, 256)));
    cusolverDnSetStream(ctx->solver, as_stream(stream));
    if (syevd_loop(N, batch)) {
        int lwork = 0;
        if ((rc = syevd_f32_lwork(ctx, N, &lwork))) return rc;
        const size_t nn = static_cast<size_t>(N) * N;
        for (int b = 0; b < batch; ++b) {
            cusolverStatus_t cs = cusolverDnSsyevd(ctx->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, N,
                                                   A + nn * b, N, evals + static_cast<size_t>(N) * b,
                                                   static_cast<float*>(work), lwork, info + b);
            if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail(cs, "cusolverDnSsyevd");
        }
        return check_cuda("cusolverDnSsyevd");
    }
    cusolverStatus_t cs = cusolverDnXsyevBatched(ctx->solver, ctx->params, CUSOLVER_EIG_MODE_VECTOR,
                                                 CUBLAS_FILL_MODE_LOWER, N, CUDA_R_32F, A, N, CUDA_R_32F, evals,
                                                 CUDA_R_32F, work, L.dev_bytes, nullptr, 0, info, batch);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail(cs, "cusolverDnXsyevBatched (FP32)");
    return check_cuda("cusolverDnXsyevBatched (FP32)");
}

// ---- covariate basis (thin SVD of X) --------------------------------------------------------------------------

namespace {

// row-major X (N, D) -> column-major copy for gesvd
__global__ void k_to_colmajor(const double* __restrict__ X, int N, int D, double* __restrict__ Xc) {
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(N) * D) return;
    int i = static_cast<int>(t / D), d = static_cast<int>(t % D);
    Xc[static_cast<int64_t>(d) * N + i] = X[t];
}

// rank by torch.linalg.pinv's default cut (sigma > eps * max(N, D) * sigma_max), the orthonormal basis rows and
// Xpinv = V diag(1 / sigma) U^T over the kept singular triplets.  S is descending (gesvd).
__global__ void k_basis_from_svd(const double* __restrict__ U, const double* __restrict__ S,
                                 const double* __restrict__ VT, int N, int D, double* __restrict__ Qx,
                                 double* __restrict__ Xpinv, int32_t* __restrict__ rank_dev) {
    const double cut = 2.220446049250313e-16 * static_cast<double>(N > D ? N : D) * S[0];
    int rank = 0;
    for (int r = 0; r < D; ++r) rank += (S[r] > cut) ? 1 : 0;
    int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t == 0) *rank_dev = rank;
    if (t >= static_cast<int64_t>(N) * D) return;
    int d = static_cast<int>(t / N), i = static_cast<int>(t % N);
    Qx[t] = (d < rank) ? U[static_cast<int64_t>(d) * N + i] : 0.0;
    double acc = 0.0;
    for (int r = 0; r < rank; ++r) acc += VT[static_cast<int64_t>(d) * D + r] * (U[static_cast<int64_t>(r) * N + i] / S[r]);
    Xpinv[t] = acc;
}

struct SvdLayout {
    size_t xc, u, s, vt, rwork, work, info, total;
    int lwork;
};

int svd_layout(flmm_context* ctx, int N, int D, SvdLayout* L) {
    int lwork = 0;
    cusolverStatus_t st = cusolverDnDgesvd_bufferSize(ctx->solver, N, D, &lwork);
    if (st != CUSOLVER_STATUS_SUCCESS) return solver_fail(st, "cusolverDnDgesvd_bufferSize");
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align_up(off + bytes, 256); return o; };
    L->xc = take(sizeof(double) * N * D);
    L->u = take(sizeof(double) * N * D);
    L->s = take(sizeof(double) * D);
    L->vt = take(sizeof(double) * D * D);
    L->rwork = take(sizeof(double) * D);
    L->work = take(sizeof(double) * static_cast<size_t>(lwork));
    L->info = take(sizeof(int));
    L->total = off;
    L->lwork = lwork;
    return FLMM_OK;
}

}  // namespace

extern "C" int flmm_covariate_basis_workspace_bytes(flmm_context* ctx, int N, int D, size_t* bytes) {
    FLMM_REQUIRE(ctx && bytes && N >= D && D > 0, "flmm_covariate_basis_workspace_bytes: need N >= D > 0");
    SvdLayout L;
    int rc = svd_layout(ctx, N, D, &L);
    if (rc) return rc;
    *bytes = L.total;
    return FLMM_OK;
}

extern "C" int flmm_covariate_basis(flmm_context* ctx, const double* X, int N, int D, double* Qx, double* Xpinv,
                                    int32_t* rank_dev, void* work, size_t work_bytes, void* stream) {
    FLMM_REQUIRE(ctx && X && Qx && Xpinv && rank_dev && work, "flmm_covariate_basis: NULL argument");
    FLMM_REQUIRE(N >= D && D > 0, "flmm_covariate_basis: need N >= D > 0 (N=%d, D=%d)", N, D);
    SvdLayout L;
    int rc = svd_layout(ctx, N, D, &L);
    if (rc) return rc;
    if (work_bytes < L.total)
        return fail(FLMM_ERR_WORKSPACE, "flmm_covariate_basis: need %zu bytes, got %zu", L.total, work_bytes);
    char* w = static_cast<char*>(work);
    double* Xc = reinterpret_cast<double*>(w + L.xc);
    double* U = reinterpret_cast<double*>(w + L.u);
    double* S = reinterpret_cast<double*>(w + L.s);
    double* VT = reinterpret_cast<double*>(w + L.vt);
    double* rwork = reinterpret_cast<double*>(w + L.rwork);
    double* dwork = reinterpret_cast<double*>(w + L.work);
    int* info = reinterpret_cast<int*>(w + L.info);
    cudaStream_t st = as_stream(stream);
    int64_t nd = static_cast<int64_t>(N) * D;
    k_to_colmajor<<<ceil_div(nd, 256), 256, 0, st>>>(X, N, D, Xc);
    if ((rc = check_launch("k_to_colmajor"))) return rc;
    cusolverDnSetStream(ctx->solver, st);
    cusolverStatus_t cs = cusolverDnDgesvd(ctx->solver, 'S', 'S', N, D, Xc, N, S, U, N, VT, D, dwork, L.lwork,
                                           rwork, info);
    if (cs != CUSOLVER_STATUS_SUCCESS) return solver_fail(cs, "cusolverDnDgesvd");
    k_basis_from_svd<<<ceil_div(nd, 256), 256, 0, st>>>(U, S, VT, N, D, Qx, Xpinv, rank_dev);
    return check_launch("k_basis_from_svd");
}
