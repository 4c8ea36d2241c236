// Training kernels of the learned delta proposal's MLP (no counterpart in the reference).
//
// The network is the one flmm_delta_mlp_f32 evaluates: 65 -> 128 -> 128 -> 1 with tanh-GELU.  Its parameters live in
// one flat FP32 array (the master weights), in this order:
//   W1 (128, 65) | b1 (128) | W2 (128, 128) | b2 (128) | w3 (128) | b3 (1)        -> FLMM_MLP_PARAMS = 25,089 floats.
//
// flmm_mlp_grad: gradient of the mean smooth-L1 loss over a minibatch (rows gathered from a feature matrix by an index
// list).  With bf16 != 0 every matrix operand is rounded to BF16 (round to nearest even) where it enters a product
// -- the inputs, the weights, the activations and the back-propagated pre-activation gradients -- and every product
// accumulates in FP32: BF16 arithmetic with FP32 master weights.  With bf16 == 0 the same kernels run on FP32 operands
// (used to check the gradient arithmetic against an FP64 restatement).  Per row:
//   z1 = W1 x + b1, a1 = gelu(z1), z2 = W2 a1 + b2, a2 = gelu(z2), o = w3 . a2 + b3,
//   loss = huber(o - y) / batch,  huber(d) = 0.5 d^2 / beta if |d| < beta else |d| - 0.5 beta,
//   g = dloss/do,  dz2 = g w3 o gelu'(z2),  dz1 = (W2^T dz2) o gelu'(z1),
//   dW2 = dz2 a1^T, dW1 = dz1 x^T, db = dz, dw3 = g a2, db3 = g.
// One CTA takes 16 rows (thread j = hidden unit j), holds both weight matrices in shared memory and writes its
// partial gradient; a second kernel adds the partials in a fixed order (deterministic, no atomics).
//
// flmm_mlp_adamw: one AdamW step on the master weights (decoupled weight decay, bias-corrected moments).
#include <math.h>

#include "flmm_common.cuh"
#include "flmm_mlp.cuh"

using namespace flmm;
using namespace flmm::mlp;

namespace {

constexpr int kRows = kMlpRows, kThreads = kMlpThreads;
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + kHid * kIn;
constexpr int OFF_W2 = OFF_B1 + kHid;
constexpr int OFF_B2 = OFF_W2 + kHid * kHid;
constexpr int OFF_W3 = OFF_B2 + kHid;
constexpr int OFF_B3 = OFF_W3 + kHid;
constexpr int kParams = OFF_B3 + 1;
static_assert(kParams == FLMM_MLP_PARAMS, "parameter layout");
constexpr int kPartialLd = (kParams + 1 + 3) / 4 * 4;  // per-CTA partial: gradient, then the loss
constexpr int LDW2 = kLdW2;

constexpr size_t kSmemFloats = static_cast<size_t>(kHid) * kIn + static_cast<size_t>(kHid) * LDW2 + kRows * kIn +
                               3 * kRows * kHid + kRows + 4 * kRows;

__global__ void __launch_bounds__(kThreads)
k_mlp_rows(const float* __restrict__ params, const float* __restrict__ X, int64_t ldx, int n_x,
           const float* __restrict__ y, const int32_t* __restrict__ rows, int batch, float huber_beta, int bf16,
           float* __restrict__ partial) {
    extern __shared__ float sm[];
    float* W1s = sm;                        // (kHid, kIn)
    float* W2s = W1s + kHid * kIn;          // (kHid, LDW2)
    float* xs = W2s + kHid * LDW2;          // (kRows, kIn)
    float* a1s = xs + kRows * kIn;          // (kRows, kHid) gelu(z1), as the products read it
    float* dz2s = a1s + kRows * kHid;       // (kRows, kHid)
    float* dz1s = dz2s + kRows * kHid;      // (kRows, kHid)
    float* gos = dz1s + kRows * kHid;       // (kRows,) dloss/do
    float* red = gos + kRows;               // (4, kRows) per-warp partial outputs

    const int j = threadIdx.x;
    auto op = [bf16](float v) { return bf16 ? round_bf16(v) : v; };
    load_weights(params + OFF_W1, params + OFF_W2, W1s, W2s, op);
    const float b1j = params[OFF_B1 + j], b2j = params[OFF_B2 + j], b3 = params[OFF_B3];
    const float w3j = op(params[OFF_W3 + j]);
    const int r0 = blockIdx.x * kRows;
    const int nr = min(kRows, batch - r0);
    for (int t = j; t < kRows * kIn; t += kThreads) {
        const int r = t / kIn, k = t % kIn;
        const int row = (r < nr) ? rows[r0 + r] : -1;
        xs[t] = (row >= 0 && row < n_x) ? op(X[static_cast<int64_t>(row) * ldx + k]) : 0.0f;
    }
    __syncthreads();

    float z1[kRows], z2[kRows], a2[kRows];
    forward_tile(W1s, W2s, xs, a1s, b1j, b2j, z1, z2, a2, op);
    output_partials(w3j, a2, red);
    __syncthreads();
    float loss = 0.0f;
    if (j < kRows) {
        float g = 0.0f;
        const int row = (j < nr) ? rows[r0 + j] : -1;
        if (row >= 0 && row < n_x) {  // an index outside the feature matrix contributes nothing
            const float o = row_output(red, j, b3);
            const float d = o - y[row];
            const float ad = fabsf(d);
            const float inv_b = 1.0f / static_cast<float>(batch);
            if (ad < huber_beta) {
                loss = 0.5f * d * d / huber_beta * inv_b;
                g = d / huber_beta * inv_b;
            } else {
                loss = (ad - 0.5f * huber_beta) * inv_b;
                g = copysignf(inv_b, d);
            }
        }
        gos[j] = g;
    }
    loss = warp_sum(loss);  // rows live in warp 0
    __syncthreads();

    // back through layer 2: dz2 of unit j, dw3, db2
    float dw3 = 0.0f, db2 = 0.0f;
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
        const float g = gos[r];
        dw3 = fmaf(g, a2[r], dw3);
        const float dz = op(g * w3j * gelu_tanh_grad(z2[r]));
        dz2s[r * kHid + j] = dz;
        db2 += dz;
    }
    __syncthreads();
    // back through W2: da1 of unit j = sum_i W2[i, j] dz2[i]
    float da1[kRows];
#pragma unroll
    for (int r = 0; r < kRows; ++r) da1[r] = 0.0f;
    for (int i = 0; i < kHid; ++i) {
        const float w = W2s[i * LDW2 + j];
#pragma unroll
        for (int r = 0; r < kRows; ++r) da1[r] = fmaf(w, dz2s[r * kHid + i], da1[r]);
    }
    float db1 = 0.0f;
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
        const float dz = op(da1[r] * gelu_tanh_grad(z1[r]));
        dz1s[r * kHid + j] = dz;
        db1 += dz;
    }
    __syncthreads();

    float* out = partial + static_cast<int64_t>(blockIdx.x) * kPartialLd;
    // dW2[u, i] = sum_r dz2[r, u] a1[r, i], dW1[u, k] = sum_r dz1[r, u] x[r, k] (flat loops: coalesced writes)
    for (int t = j; t < kHid * kHid; t += kThreads) {
        const int u = t / kHid, i = t % kHid;
        float acc = 0.0f;
#pragma unroll
        for (int r = 0; r < kRows; ++r) acc = fmaf(dz2s[r * kHid + u], a1s[r * kHid + i], acc);
        out[OFF_W2 + t] = acc;
    }
    for (int t = j; t < kHid * kIn; t += kThreads) {
        const int u = t / kIn, k = t % kIn;
        float acc = 0.0f;
#pragma unroll
        for (int r = 0; r < kRows; ++r) acc = fmaf(dz1s[r * kHid + u], xs[r * kIn + k], acc);
        out[OFF_W1 + t] = acc;
    }
    out[OFF_B1 + j] = db1;
    out[OFF_B2 + j] = db2;
    out[OFF_W3 + j] = dw3;
    if (j == 0) {
        float g = 0.0f;
        for (int r = 0; r < kRows; ++r) g += gos[r];
        out[OFF_B3] = g;
        out[kParams] = loss;
    }
}

// grad[p] = sum over CTAs of the partials, in CTA order; loss (if given) likewise
__global__ void k_mlp_reduce(const float* __restrict__ partial, int n_parts, float* __restrict__ grad,
                             float* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > kParams) return;
    float acc = 0.0f;
    for (int c = 0; c < n_parts; ++c) acc += partial[static_cast<int64_t>(c) * kPartialLd + p];
    if (p < kParams) grad[p] = acc;
    else if (loss) *loss = acc;
}

// AdamW (decoupled weight decay): w -= lr wd w; m, v moments; w -= lr mhat / (sqrt(vhat) + eps)
__global__ void k_mlp_adamw(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int n, float lr, float beta1, float beta2, float eps, float wd,
                            float bc1, float bc2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float gp = g[p];
    float wp = w[p] * (1.0f - lr * wd);
    const float mp = beta1 * m[p] + (1.0f - beta1) * gp;
    const float vp = beta2 * v[p] + (1.0f - beta2) * gp * gp;
    m[p] = mp;
    v[p] = vp;
    wp -= lr * (mp / bc1) / (sqrtf(vp / bc2) + eps);
    w[p] = wp;
}

unsigned n_row_blocks(int batch) { return ceil_div(batch, kRows); }

}  // namespace

extern "C" int flmm_mlp_grad_workspace_bytes(int batch, size_t* bytes) {
    FLMM_REQUIRE(bytes && batch > 0, "flmm_mlp_grad_workspace_bytes: bad arguments");
    *bytes = sizeof(float) * static_cast<size_t>(kPartialLd) * n_row_blocks(batch);
    return FLMM_OK;
}

extern "C" int flmm_mlp_grad(const float* params, const float* X, int64_t ldx, int n_x, const float* y,
                             const int32_t* rows, int batch, float huber_beta, int bf16, float* grad, float* loss,
                             void* work, size_t work_bytes, void* stream) {
    FLMM_REQUIRE(params && X && y && rows && grad && work && batch > 0 && n_x > 0 && ldx >= kIn && huber_beta > 0.0f,
                 "flmm_mlp_grad: bad arguments (X rows hold %d features; huber_beta > 0)", kIn);
    size_t need = 0;
    int rc = flmm_mlp_grad_workspace_bytes(batch, &need);
    if (rc) return rc;
    if (work_bytes < need) return fail(FLMM_ERR_WORKSPACE, "flmm_mlp_grad: need %zu bytes, got %zu", need, work_bytes);
    cudaStream_t st = as_stream(stream);
    const size_t smem = sizeof(float) * kSmemFloats;
    FLMM_CUDA(cudaFuncSetAttribute(k_mlp_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    float* partial = static_cast<float*>(work);
    const unsigned blocks = n_row_blocks(batch);
    k_mlp_rows<<<blocks, kThreads, smem, st>>>(params, X, ldx, n_x, y, rows, batch, huber_beta, bf16, partial);
    if ((rc = check_launch("k_mlp_rows"))) return rc;
    k_mlp_reduce<<<ceil_div(kParams + 1, 256), 256, 0, st>>>(partial, static_cast<int>(blocks), grad, loss);
    return check_launch("k_mlp_reduce");
}

extern "C" int flmm_mlp_adamw(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1,
                              float beta2, float eps, float weight_decay, void* stream) {
    FLMM_REQUIRE(params && grad && m && v && step >= 1 && beta1 >= 0.0f && beta1 < 1.0f && beta2 >= 0.0f &&
                     beta2 < 1.0f && eps > 0.0f,
                 "flmm_mlp_adamw: bad arguments (step counts from 1)");
    const float bc1 = static_cast<float>(1.0 - pow(static_cast<double>(beta1), step));
    const float bc2 = static_cast<float>(1.0 - pow(static_cast<double>(beta2), step));
    k_mlp_adamw<<<ceil_div(kParams, 256), 256, 0, as_stream(stream)>>>(params, grad, m, v, kParams, lr, beta1, beta2,
                                                                       eps, weight_decay, bc1, bc2);
    return check_launch("k_mlp_adamw");
}
