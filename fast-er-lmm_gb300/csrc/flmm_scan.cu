// Scan-level C ABI of the fast form: the whole LOCO permutation scan (fasterlmm/perms.py:21-68 ->
// fasterlmm/core.py:677-726) driven from native code, for callers that do not go through Python.
//
//   flmm_scan_create / flmm_scan_destroy   a scan object bound to one device: its library context, a second stream
//                                          for the column side, and the device buffers it owns
//   flmm_scan_group_prepare                covariates and kinship panel of one sample group: the covariate basis,
//                                          per-chromosome Grams (split-FP16 tensor-core products), the LOCO kinships
//                                          projected off the covariates, their batched FP32 eigendecomposition and
//                                          refinement against the FP64 kinships -> per-chromosome spectra
//   flmm_scan_rotate_phenos                the scan columns (reals and permutations) regressed off the covariates and
//                                          split for the tensor cores
//   flmm_scan_fit_delta                    one chromosome's column side: UY = U_eff^T Y_r and the delta fit
//   flmm_scan_wald                         one chromosome's variant side: US = U_eff^T S_r, the fused Wald scan and
//                                          the re-evaluation of its strong real tests
//   flmm_scan_run                          every chromosome, the column side of chromosome k + 1 on the second
//                                          stream while the variant side of chromosome k runs on the caller's stream
//
// Inputs and outputs are caller-owned device pointers; every call takes a stream and returns a status.  The object
// allocates its working buffers (cudaMalloc) when it first needs them and keeps them for later calls of the same or
// smaller sizes.  A scan object is used by one host thread at a time.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "flmm_common.cuh"

using namespace flmm;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    int ensure(size_t bytes) {
        if (bytes <= n && p) return FLMM_OK;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        const size_t b = bytes < 256 ? 256 : bytes;
        if (cudaMalloc(&p, b) != cudaSuccess) {
            cudaGetLastError();
            return fail(FLMM_ERR_CUDA, "flmm_scan: cannot allocate %zu bytes of device memory", b);
        }
        n = b;
        return FLMM_OK;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

struct Split {  // hi / lo FP16 rows with a power-of-two scale per row
    DevBuf hi, lo, scale;
    int64_t ld = 0;
    int ensure(int rows, int64_t ld_) {
        ld = ld_;
        int rc;
        if ((rc = hi.ensure(2 * static_cast<size_t>(rows) * ld))) return rc;
        if ((rc = lo.ensure(2 * static_cast<size_t>(rows) * ld))) return rc;
        return scale.ensure(4 * static_cast<size_t>(rows));
    }
};

inline int64_t pad8(int64_t k) { return (k + 7) / 8 * 8; }

constexpr double kInterpH = 0.25;  // sWs interpolation nodes in log delta (see flmm_wald_split_prep_columns)
constexpr int kInterpQ = 10;
constexpr int kRefineCap = 1 << 22;

__global__ void k_gather_rows_f64(const double* __restrict__ src, int64_t lds, const int64_t* __restrict__ idx,
                                  int rows, int N, double* __restrict__ dst, int64_t ldd) {
    const int r = blockIdx.y;
    if (r >= rows) return;
    const double* s = src + idx[r] * lds;
    double* d = dst + static_cast<int64_t>(r) * ldd;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) d[i] = s[i];
}

struct ColumnSlot {  // one chromosome's column side, two of them alternate
    Split Us;        // U_eff rows (Neff, N), split
    DevBuf UY;       // (P, ldk) FP32
    DevBuf ld;       // (P,) log delta
    DevBuf idx;      // (P,) grid argmin
    DevBuf work;     // delta-fit workspace
};

}  // namespace

struct flmm_scan {
    int device = 0;
    flmm_context* ctx = nullptr;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_start = nullptr, ev_ready[2] = {}, ev_free[2] = {};
    int N = 0, D = 0, Neff = 0;
    int64_t ldN = 0, ldk = 0;
    flmm_scan_opts opts{};
    // covariates
    DevBuf X, Qx, Xpinv, rank;
    // prepared chromosomes (units): LOCO chromosome ids, FP64 kinships -> FP32 eigenvector rows, spectra
    int n_units = 0;
    std::vector<int32_t> unit_chrom;
    std::vector<char> unit_all;  // 1: kinship of the whole panel (single-K)
    DevBuf Kp, U, U2, evals64, s, s32all;
    // phenotypes
    int P = 0;
    Split Ys;
    // column side slots and variant side buffers
    ColumnSlot slot[2];
    DevBuf rows_all, USt, flags, flag_count, shat, s32, W, F;
    Split Zs, Ws, Fs;
    DevBuf A1h, A1l, Lh, Ll, sa1, sl, rWr, rWr0, B1h, B1l, B2h, B2l, sb1, sb2;
    DevBuf work;
};

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int split_rows(const void* X, int is_f64, int64_t ldx, int rows, int K, Split& out, int64_t ld, cudaStream_t st) {
    int rc = out.ensure(rows, ld);
    if (rc || rows == 0) return rc;
    return flmm_split_rows_f16(X, is_f64, ldx, rows, K, out.hi.p, out.lo.p, ld, out.scale.as<float>(), st);
}

int interp_R(double lo, double hi, double* x0) {
    *x0 = lo - (kInterpQ / 2) * kInterpH;
    return static_cast<int>(std::ceil((hi - lo) / kInterpH - 1e-9)) + kInterpQ + 1;
}

int refine_steps(const flmm_scan& s) {
    if (s.opts.eigh_refine_steps > 0) return s.opts.eigh_refine_steps;
    return s.N <= 1024 ? 2 : 3;
}

// Column side of unit u into slot b: U_eff split, UY rotation, delta fit (stream st).
int column_side(flmm_scan& s, int u, int b, cudaStream_t st) {
    ColumnSlot& cs = s.slot[b];
    int rc;
    const float* Uu = s.U.as<float>() + static_cast<int64_t>(u) * s.N * s.N;
    if ((rc = split_rows(Uu + static_cast<int64_t>(s.D) * s.N, 0, s.N, s.Neff, s.N, cs.Us, s.ldN, st))) return rc;
    if ((rc = cs.UY.ensure(4 * static_cast<size_t>(s.P) * s.ldk))) return rc;
    if ((rc = cs.ld.ensure(8 * static_cast<size_t>(s.P)))) return rc;
    if ((rc = cs.idx.ensure(4 * static_cast<size_t>(s.P)))) return rc;
    if (s.P == 0) return FLMM_OK;
    if ((rc = flmm_gemm_split_f16(s.ctx, s.Ys.hi.p, s.Ys.lo.p, s.Ys.scale.as<float>(), s.Ys.ld, s.P, cs.Us.hi.p,
                                  cs.Us.lo.p, cs.Us.scale.as<float>(), cs.Us.ld, s.Neff, s.N, cs.UY.as<float>(), s.ldk,
                                  0, st)))
        return rc;
    size_t wb = 0;
    if ((rc = flmm_fit_delta_fast_workspace_bytes(s.Neff, s.opts.n_grid, &wb))) return rc;
    if ((rc = cs.work.ensure(wb))) return rc;
    return flmm_fit_delta_fast(s.s.as<double>() + static_cast<int64_t>(u) * s.Neff, s.Neff, cs.UY.as<float>(),
                               s.ldk, s.P, s.opts.n_grid, s.opts.log_delta_min, s.opts.log_delta_max, s.opts.refine,
                               cs.ld.as<double>(), cs.idx.as<int32_t>(), cs.work.p, cs.work.n, st);
}

// Variant side of unit u with its column side in slot b: Zt_c (Mc, N) standardised variants of the chromosome.
int variant_side(flmm_scan& s, int u, int b, const double* Zt_c, int64_t ldz, int Mc, const int64_t* rows,
                 int n_real, double* f, double* beta, double* se, double* sfve, double* nullh2, int64_t ldo,
                 double* max_F, cudaStream_t st) {
    if (Mc == 0) return FLMM_OK;
    ColumnSlot& cs = s.slot[b];
    const int N = s.N, Neff = s.Neff, P = s.P;
    const int64_t ldk = s.ldk;
    int rc;
    // US = U_eff^T S_r = U_eff^T S: the kept eigenvectors are orthogonal to the covariates, so the variants need no
    // regressing off (fasterlmm/core.py:628-629)
    if ((rc = split_rows(Zt_c, 1, ldz, Mc, N, s.Zs, s.ldN, st))) return rc;
    if ((rc = s.USt.ensure(4 * static_cast<size_t>(Mc) * ldk))) return rc;
    if ((rc = flmm_gemm_split_f16(s.ctx, s.Zs.hi.p, s.Zs.lo.p, s.Zs.scale.as<float>(), s.Zs.ld, Mc, cs.Us.hi.p,
                                  cs.Us.lo.p, cs.Us.scale.as<float>(), cs.Us.ld, Neff, N, s.USt.as<float>(), ldk, 0,
                                  st)))
        return rc;
    if (P == 0) return FLMM_OK;
    // Wald operands (the steps of fasterlmm_gb300.fast.wald_fast)
    double x0 = 0.0;
    const int R = interp_R(s.opts.log_delta_min, s.opts.log_delta_max, &x0);
    const int64_t ldr = pad8(R);
    const double* su = s.s.as<double>() + static_cast<int64_t>(u) * Neff;
    if ((rc = s.s32.ensure(4 * static_cast<size_t>(Neff)))) return rc;
    if ((rc = s.shat.ensure(4))) return rc;
    if ((rc = flmm_convert_f64_f32(Neff, su, s.s32.as<float>(), st))) return rc;
    if ((rc = flmm_mean_f32(su, Neff, s.shat.as<float>(), st))) return rc;
    const size_t P2k = 2 * static_cast<size_t>(P) * ldk, P2r = 2 * static_cast<size_t>(P) * ldr;
    if ((rc = s.A1h.ensure(P2k)) || (rc = s.A1l.ensure(P2k)) || (rc = s.Lh.ensure(P2r)) || (rc = s.Ll.ensure(P2r)) ||
        (rc = s.sa1.ensure(4 * static_cast<size_t>(P))) || (rc = s.sl.ensure(4 * static_cast<size_t>(P))) ||
        (rc = s.rWr.ensure(4 * static_cast<size_t>(P))) || (rc = s.rWr0.ensure(4 * static_cast<size_t>(P))))
        return rc;
    if ((rc = flmm_wald_split_prep_columns(s.s32.as<float>(), Neff, cs.UY.as<float>(), ldk, cs.ld.as<double>(), P,
                                           s.shat.as<float>(), x0, kInterpH, R, s.A1h.p, s.A1l.p, ldk, s.Lh.p,
                                           s.Ll.p, ldr, s.sa1.as<float>(), s.sl.as<float>(), s.rWr.as<float>(),
                                           s.rWr0.as<float>(), st)))
        return rc;
    const size_t M2k = 2 * static_cast<size_t>(Mc) * ldk;
    if ((rc = s.B1h.ensure(M2k)) || (rc = s.B1l.ensure(M2k)) || (rc = s.B2h.ensure(M2k)) || (rc = s.B2l.ensure(M2k)) ||
        (rc = s.sb1.ensure(4 * static_cast<size_t>(Mc))) || (rc = s.sb2.ensure(4 * static_cast<size_t>(Mc))))
        return rc;
    if ((rc = flmm_wald_split_prep_variants(s.USt.as<float>(), ldk, Mc, Neff, s.B1h.p, s.B1l.p, s.B2h.p, s.B2l.p, ldk,
                                            s.sb1.as<float>(), s.sb2.as<float>(), st)))
        return rc;
    // node values of sWs~: F (Mc, R) = (US o US) W~^T
    if ((rc = s.W.ensure(8 * static_cast<size_t>(R) * Neff))) return rc;
    if ((rc = flmm_wald_interp_nodes(su, Neff, s.shat.as<float>(), x0, kInterpH, R, s.W.as<double>(), st))) return rc;
    if ((rc = split_rows(s.W.p, 1, Neff, R, Neff, s.Ws, ldk, st))) return rc;
    if ((rc = s.F.ensure(4 * static_cast<size_t>(Mc) * ldr))) return rc;
    if ((rc = flmm_gemm_split_f16(s.ctx, s.B2h.p, s.B2l.p, s.sb2.as<float>(), ldk, Mc, s.Ws.hi.p, s.Ws.lo.p,
                                  s.Ws.scale.as<float>(), s.Ws.ld, R, Neff, s.F.as<float>(), ldr, 0, st)))
        return rc;
    if ((rc = split_rows(s.F.p, 0, ldr, Mc, R, s.Fs, ldr, st))) return rc;
    // fused Wald with the strong-test list, then the re-evaluation
    const bool refine = s.opts.f_refine > 0.0 && n_real > 0;
    const int cap = refine ? static_cast<int>(std::min<int64_t>(static_cast<int64_t>(Mc) * n_real, kRefineCap)) : 0;
    if ((rc = s.flags.ensure(8 * static_cast<size_t>(cap > 0 ? cap : 1)))) return rc;
    if ((rc = s.flag_count.ensure(4))) return rc;
    const float fcut = refine ? static_cast<float>(s.opts.f_refine) : INFINITY;
    if ((rc = flmm_wald_split_f16(s.ctx, s.A1h.p, s.A1l.p, ldk, s.sa1.as<float>(), s.Lh.p, s.Ll.p, ldr,
                                  s.sl.as<float>(), s.rWr.as<float>(), s.rWr0.as<float>(), P, n_real, s.B1h.p,
                                  s.B1l.p, ldk, s.sb1.as<float>(), s.Fs.hi.p, s.Fs.lo.p, s.Fs.ld,
                                  s.Fs.scale.as<float>(), Mc, Neff, R, rows, f, beta, se, sfve, ldo, max_F, fcut,
                                  refine ? s.flag_count.as<int32_t>() : nullptr,
                                  refine ? s.flags.as<int32_t>() : nullptr, cap, st)))
        return rc;
    if (refine &&
        (rc = flmm_wald_refine_f32(s.ctx, s.flags.as<int32_t>(), s.flag_count.as<int32_t>(), cap, fcut,
                                   s.USt.as<float>(), ldk, cs.UY.as<float>(), ldk, s.s32.as<float>(),
                                   cs.ld.as<double>(), Neff, Mc, n_real, rows, f, beta, se, sfve, ldo, max_F, st)))
        return rc;
    if (nullh2 && n_real > 0)
        return flmm_fill_nullh2(cs.ld.as<double>(), n_real, rows, Mc, nullh2, ldo, st);
    return FLMM_OK;
}

}  // namespace

extern "C" int flmm_scan_opts_default(flmm_scan_opts* o) {
    FLMM_REQUIRE(o, "flmm_scan_opts_default: null pointer");
    o->n_grid = 64;
    o->log_delta_min = -10.0;
    o->log_delta_max = 10.0;
    o->refine = 1;
    o->eigh_refine_steps = 0;
    o->f_refine = 30.0;
    o->pipeline = 1;
    return FLMM_OK;
}

extern "C" int flmm_scan_create(int device, int N, int D, const flmm_scan_opts* opts, flmm_scan** out) {
    FLMM_REQUIRE(out && N > D && D >= 1 && N >= 3, "flmm_scan_create: need N > D >= 1 (N = %d, D = %d)", N, D);
    *out = nullptr;
    flmm_scan_opts o;
    flmm_scan_opts_default(&o);
    if (opts) o = *opts;
    FLMM_REQUIRE(o.n_grid >= 1 && o.log_delta_max > o.log_delta_min, "flmm_scan_create: bad delta grid");
    DeviceGuard g(device);
    flmm_scan* s = new (std::nothrow) flmm_scan();
    if (!s) return fail(FLMM_ERR_ARG, "flmm_scan_create: out of host memory");
    s->device = device;
    s->N = N;
    s->D = D;
    s->Neff = N - D;
    s->ldN = pad8(N);
    s->ldk = pad8(N - D);
    s->opts = o;
    int rc = flmm_context_create(device, &s->ctx);
    if (!rc && cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) != cudaSuccess)
        rc = fail(FLMM_ERR_CUDA, "flmm_scan_create: cannot create a stream");
    cudaEvent_t* evs[] = {&s->ev_start, &s->ev_ready[0], &s->ev_ready[1], &s->ev_free[0], &s->ev_free[1]};
    for (cudaEvent_t* e : evs)
        if (!rc && cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess)
            rc = fail(FLMM_ERR_CUDA, "flmm_scan_create: cannot create an event");
    if (rc) {
        flmm_scan_destroy(s);
        return rc;
    }
    *out = s;
    return FLMM_OK;
}

extern "C" int flmm_scan_destroy(flmm_scan* s) {
    if (!s) return FLMM_OK;
    DeviceGuard g(s->device);
    if (s->side) cudaStreamSynchronize(s->side);
    cudaDeviceSynchronize();
    cudaEvent_t evs[] = {s->ev_start, s->ev_ready[0], s->ev_ready[1], s->ev_free[0], s->ev_free[1]};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    if (s->side) cudaStreamDestroy(s->side);
    if (s->ctx) flmm_context_destroy(s->ctx);
    delete s;
    return FLMM_OK;
}

extern "C" int flmm_scan_group_prepare(flmm_scan* s, const double* X, const double* Zt_kin, int64_t ldz, int M_kin,
                                       const int32_t* chrom_kin, const int32_t* loco_chroms, int n_units,
                                       void* stream) {
    FLMM_REQUIRE(s && X && Zt_kin && chrom_kin && M_kin > 0 && ldz >= s->N && n_units >= 0 && (loco_chroms || n_units == 0),
                 "flmm_scan_group_prepare: bad arguments");
    DeviceGuard g(s->device);
    cudaStream_t st = as_stream(stream);
    const int N = s->N, D = s->D;
    int rc;
    // covariates: a private copy of X, its basis and pseudo-inverse
    if ((rc = s->X.ensure(8 * static_cast<size_t>(N) * D)) || (rc = s->Qx.ensure(8 * static_cast<size_t>(N) * D)) ||
        (rc = s->Xpinv.ensure(8 * static_cast<size_t>(N) * D)) || (rc = s->rank.ensure(4)))
        return rc;
    FLMM_CUDA(cudaMemcpyAsync(s->X.p, X, 8 * static_cast<size_t>(N) * D, cudaMemcpyDeviceToDevice, st));
    size_t wb = 0;
    if ((rc = flmm_covariate_basis_workspace_bytes(s->ctx, N, D, &wb)) || (rc = s->work.ensure(wb))) return rc;
    if ((rc = flmm_covariate_basis(s->ctx, s->X.as<double>(), N, D, s->Qx.as<double>(), s->Xpinv.as<double>(),
                                   s->rank.as<int32_t>(), s->work.p, s->work.n, st)))
        return rc;
    // kinship panel: chromosomes in ascending order, each a 64-aligned column block of the sample-major split panel
    std::vector<int32_t> cs(chrom_kin, chrom_kin + M_kin);
    std::vector<int64_t> order(M_kin);
    for (int64_t i = 0; i < M_kin; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return cs[a] < cs[b]; });
    std::vector<int32_t> ids;
    std::vector<int64_t> starts, counts, offs;
    int64_t Mpad = 0;
    for (int64_t i = 0; i < M_kin; ++i) {
        if (ids.empty() || cs[order[i]] != ids.back()) {
            ids.push_back(cs[order[i]]);
            starts.push_back(i);
            counts.push_back(0);
            offs.push_back(Mpad);
        }
        ++counts.back();
        if (i + 1 == M_kin || cs[order[i + 1]] != ids.back()) Mpad += (counts.back() + 63) / 64 * 64;
    }
    DevBuf idx, Zsorted, Zg, Gtot, Gc;
    if ((rc = idx.ensure(8 * static_cast<size_t>(M_kin)))) return rc;
    FLMM_CUDA(cudaMemcpyAsync(idx.p, order.data(), 8 * static_cast<size_t>(M_kin), cudaMemcpyHostToDevice, st));
    if ((rc = Zsorted.ensure(8 * static_cast<size_t>(M_kin) * N))) return rc;
    k_gather_rows_f64<<<dim3(ceil_div(N, 256), M_kin), 256, 0, st>>>(Zt_kin, ldz, idx.as<int64_t>(), M_kin, N,
                                                                     Zsorted.as<double>(), N);
    if ((rc = check_launch("k_gather_rows_f64"))) return rc;
    if ((rc = Zg.ensure(8 * static_cast<size_t>(N) * Mpad))) return rc;
    FLMM_CUDA(cudaMemsetAsync(Zg.p, 0, 8 * static_cast<size_t>(N) * Mpad, st));
    for (size_t c = 0; c < ids.size(); ++c)
        if ((rc = flmm_transpose_f64(Zsorted.as<double>() + starts[c] * N, N, static_cast<int>(counts[c]), N,
                                     Zg.as<double>() + offs[c], Mpad, st)))
            return rc;
    Split Kz;
    if ((rc = split_rows(Zg.p, 1, Mpad, N, static_cast<int>(Mpad), Kz, Mpad, st))) return rc;
    // per-chromosome Grams and their FP64 total
    if ((rc = Gtot.ensure(8 * static_cast<size_t>(N) * N))) return rc;
    FLMM_CUDA(cudaMemsetAsync(Gtot.p, 0, 8 * static_cast<size_t>(N) * N, st));
    if ((rc = Gc.ensure(4 * static_cast<size_t>(N) * N * ids.size()))) return rc;
    for (size_t c = 0; c < ids.size(); ++c) {
        float* G = Gc.as<float>() + static_cast<int64_t>(c) * N * N;
        const uint16_t* hi = static_cast<const uint16_t*>(Kz.hi.p) + offs[c];
        const uint16_t* lo = static_cast<const uint16_t*>(Kz.lo.p) + offs[c];
        if ((rc = flmm_gemm_split_f16(s->ctx, hi, lo, Kz.scale.as<float>(), Mpad, N, hi, lo, Kz.scale.as<float>(),
                                      Mpad, N, static_cast<int>(counts[c]), G, N, 0, st)))
            return rc;
        if ((rc = flmm_accumulate_f32_f64(static_cast<int64_t>(N) * N, G, Gtot.as<double>(), st))) return rc;
    }
    // LOCO kinships, projected off the covariates; a unit whose chromosome is not in the panel (or single-K,
    // n_units == 0) uses the whole panel
    const int nu = n_units > 0 ? n_units : 1;
    s->n_units = nu;
    s->unit_chrom.assign(nu, 0);
    s->unit_all.assign(nu, 1);
    const size_t nn = static_cast<size_t>(N) * N;
    if ((rc = s->Kp.ensure(8 * nn * nu)) || (rc = s->U.ensure(4 * nn * nu)) || (rc = s->U2.ensure(4 * nn * nu)) ||
        (rc = s->evals64.ensure(8 * static_cast<size_t>(N) * nu)) ||
        (rc = s->s.ensure(8 * static_cast<size_t>(s->Neff) * nu)) || (rc = s->s32all.ensure(4 * static_cast<size_t>(N) * nu)))
        return rc;
    DevBuf K;
    if ((rc = K.ensure(8 * nn))) return rc;
    if ((rc = flmm_project_kinship_workspace_bytes(N, D, &wb)) || (rc = s->work.ensure(wb))) return rc;
    for (int u = 0; u < nu; ++u) {
        const float* Gu = nullptr;
        int64_t m_loco = M_kin;
        if (n_units > 0) {
            s->unit_chrom[u] = loco_chroms[u];
            for (size_t c = 0; c < ids.size(); ++c)
                if (ids[c] == loco_chroms[u]) {
                    Gu = Gc.as<float>() + static_cast<int64_t>(c) * N * N;
                    m_loco -= counts[c];
                    s->unit_all[u] = 0;
                }
        }
        FLMM_REQUIRE(m_loco > 0, "flmm_scan_group_prepare: chromosome %d holds every kinship variant", loco_chroms[u]);
        if ((rc = flmm_loco_kinship_f32(Gtot.as<double>(), Gu, N, static_cast<double>(m_loco), K.as<double>(), st)))
            return rc;
        if ((rc = flmm_project_kinship(K.as<double>(), N, s->Qx.as<double>(), N, D, s->Kp.as<double>() + u * nn, N,
                                       s->work.p, s->work.n, st)))
            return rc;
    }
    // batched FP32 eigendecomposition, refined against the FP64 kinships
    if ((rc = flmm_convert_f64_f32(static_cast<int64_t>(nn) * nu, s->Kp.as<double>(), s->U.as<float>(), st))) return rc;
    if ((rc = flmm_eigh_batched_f32_workspace_bytes(s->ctx, N, nu, &wb)) || (rc = s->work.ensure(wb))) return rc;
    if ((rc = flmm_eigh_batched_f32(s->ctx, s->U.as<float>(), N, nu, s->s32all.as<float>(), s->work.p, s->work.n, st)))
        return rc;
    if ((rc = flmm_eigh_refine_workspace_bytes(N, nu, &wb)) || (rc = s->work.ensure(wb))) return rc;
    for (int step = 0; step < refine_steps(*s); ++step) {
        if ((rc = flmm_eigh_refine_f32(s->Kp.as<double>(), s->U.as<float>(), s->U2.as<float>(),
                                       s->evals64.as<double>(), N, nu, s->work.p, s->work.n, st)))
            return rc;
        std::swap(s->U.p, s->U2.p);
        std::swap(s->U.n, s->U2.n);
    }
    for (int u = 0; u < nu; ++u)
        if ((rc = flmm_compat_spectrum(s->evals64.as<double>() + static_cast<int64_t>(u) * N, N, D,
                                       s->s.as<double>() + static_cast<int64_t>(u) * s->Neff, st)))
            return rc;
    // the temporary buffers above are freed when this call returns: wait for the work that reads them
    FLMM_CUDA(cudaStreamSynchronize(st));
    return flmm_context_check(s->ctx, stream);
}

extern "C" int flmm_scan_rotate_phenos(flmm_scan* s, const double* Yt, int64_t ldy, int P, void* stream) {
    FLMM_REQUIRE(s && P >= 0 && (Yt || P == 0) && ldy >= s->N && s->X.p, "flmm_scan_rotate_phenos: bad arguments "
                 "(group_prepare first)");
    DeviceGuard g(s->device);
    cudaStream_t st = as_stream(stream);
    s->P = P;
    if (P == 0) return FLMM_OK;
    DevBuf Yr;
    int rc;
    if ((rc = Yr.ensure(8 * static_cast<size_t>(P) * s->N))) return rc;
    if ((rc = flmm_regress_out(Yt, ldy, P, s->N, s->X.as<double>(), s->D, s->Xpinv.as<double>(), Yr.as<double>(), s->N,
                               st)))
        return rc;
    if ((rc = split_rows(Yr.p, 1, s->N, P, s->N, s->Ys, s->ldN, st))) return rc;
    FLMM_CUDA(cudaStreamSynchronize(st));  // Yr is freed on return
    return FLMM_OK;
}

extern "C" int flmm_scan_fit_delta(flmm_scan* s, int unit, double* log_delta_out, void* stream) {
    FLMM_REQUIRE(s && unit >= 0 && unit < s->n_units, "flmm_scan_fit_delta: bad unit");
    DeviceGuard g(s->device);
    cudaStream_t st = as_stream(stream);
    int rc = column_side(*s, unit, unit & 1, st);
    if (rc) return rc;
    if (log_delta_out && s->P > 0)
        FLMM_CUDA(cudaMemcpyAsync(log_delta_out, s->slot[unit & 1].ld.p, 8 * static_cast<size_t>(s->P),
                                  cudaMemcpyDeviceToDevice, st));
    return FLMM_OK;
}

extern "C" int flmm_scan_wald(flmm_scan* s, int unit, const double* Zt_c, int64_t ldz, int Mc, const int64_t* rows,
                              int n_real, double* f, double* beta, double* se, double* sfve, double* nullh2,
                              int64_t ldo, double* max_F, void* stream) {
    FLMM_REQUIRE(s && unit >= 0 && unit < s->n_units && Mc >= 0 && (Zt_c || Mc == 0) && ldz >= s->N && n_real >= 0 &&
                     n_real <= s->P && max_F && (n_real == 0 || Mc == 0 || (rows && f && beta && se && sfve && ldo >= n_real)),
                 "flmm_scan_wald: bad arguments");
    DeviceGuard g(s->device);
    return variant_side(*s, unit, unit & 1, Zt_c, ldz, Mc, rows, n_real, f, beta, se, sfve, nullh2, ldo, max_F,
                        as_stream(stream));
}

extern "C" int flmm_scan_run(flmm_scan* s, const double* Zt, int64_t ldz, int M, const int32_t* chrom, int n_real,
                             double* f, double* beta, double* se, double* sfve, double* nullh2, int64_t ldo,
                             double* max_F, double* log_delta_out, void* stream) {
    FLMM_REQUIRE(s && M >= 0 && (Zt || M == 0) && (chrom || M == 0) && ldz >= s->N && n_real >= 0 && n_real <= s->P &&
                     max_F && s->n_units > 0 && (n_real == 0 || M == 0 || (f && beta && se && sfve && ldo >= n_real)),
                 "flmm_scan_run: bad arguments (group_prepare and rotate_phenos first)");
    DeviceGuard g(s->device);
    cudaStream_t main = as_stream(stream);
    const int nu = s->n_units;
    // tested variants of each unit: the unit's chromosome (LOCO), or all variants (a whole-panel unit)
    std::vector<std::vector<int64_t>> sel(nu);
    for (int u = 0; u < nu; ++u) {
        if (s->unit_all[u] && nu == 1) {
            sel[u].resize(M);
            for (int64_t m = 0; m < M; ++m) sel[u][m] = m;
        } else {
            for (int64_t m = 0; m < M; ++m)
                if (chrom[m] == s->unit_chrom[u]) sel[u].push_back(m);
        }
    }
    int64_t total = 0, mc_max = 0;
    for (auto& v : sel) {
        total += static_cast<int64_t>(v.size());
        mc_max = std::max<int64_t>(mc_max, static_cast<int64_t>(v.size()));
    }
    std::vector<int64_t> rows_h;
    rows_h.reserve(total);
    for (auto& v : sel) rows_h.insert(rows_h.end(), v.begin(), v.end());
    int rc;
    if ((rc = s->rows_all.ensure(8 * static_cast<size_t>(total > 0 ? total : 1)))) return rc;
    DevBuf Zblock;
    if ((rc = Zblock.ensure(8 * static_cast<size_t>(mc_max > 0 ? mc_max : 1) * s->N))) return rc;
    if (total)
        FLMM_CUDA(cudaMemcpyAsync(s->rows_all.p, rows_h.data(), 8 * static_cast<size_t>(total), cudaMemcpyHostToDevice,
                                  main));
    if ((rc = flmm_fill_f64(max_F, s->P, -INFINITY, main))) return rc;
    const bool pipe = s->opts.pipeline != 0;
    cudaStream_t side = pipe ? s->side : main;
    if (pipe) {
        FLMM_CUDA(cudaEventRecord(s->ev_start, main));
        FLMM_CUDA(cudaStreamWaitEvent(side, s->ev_start, 0));
    }
    bool used[2] = {false, false};
    auto issue_column = [&](int u) -> int {
        const int b = u & 1;
        if (pipe && used[b]) {
            int r2 = cudaStreamWaitEvent(side, s->ev_free[b], 0) == cudaSuccess ? FLMM_OK
                                                                                   : fail(FLMM_ERR_CUDA, "event wait");
            if (r2) return r2;
        }
        int r2 = column_side(*s, u, b, side);
        if (r2) return r2;
        if (log_delta_out && s->P > 0 &&
            cudaMemcpyAsync(log_delta_out + static_cast<int64_t>(u) * s->P, s->slot[b].ld.p,
                            8 * static_cast<size_t>(s->P), cudaMemcpyDeviceToDevice, side) != cudaSuccess)
            return fail(FLMM_ERR_CUDA, "flmm_scan_run: log delta copy");
        if (pipe && cudaEventRecord(s->ev_ready[b], side) != cudaSuccess) return fail(FLMM_ERR_CUDA, "event record");
        used[b] = true;
        return FLMM_OK;
    };
    if ((rc = issue_column(0))) return rc;
    int64_t off = 0;
    for (int u = 0; u < nu; ++u) {
        if (u + 1 < nu && (rc = issue_column(u + 1))) return rc;
        const int b = u & 1;
        if (pipe) FLMM_CUDA(cudaStreamWaitEvent(main, s->ev_ready[b], 0));
        const int Mc = static_cast<int>(sel[u].size());
        if (Mc) {
            k_gather_rows_f64<<<dim3(ceil_div(s->N, 256), Mc), 256, 0, main>>>(
                Zt, ldz, s->rows_all.as<int64_t>() + off, Mc, s->N, Zblock.as<double>(), s->N);
            if ((rc = check_launch("k_gather_rows_f64"))) return rc;
            if ((rc = variant_side(*s, u, b, Zblock.as<double>(), s->N, Mc, s->rows_all.as<int64_t>() + off, n_real, f,
                                   beta, se, sfve, nullh2, ldo, max_F, main)))
                return rc;
        }
        if (pipe) FLMM_CUDA(cudaEventRecord(s->ev_free[b], main));
        off += Mc;
    }
    FLMM_CUDA(cudaStreamSynchronize(main));  // Zblock is freed on return; also surfaces a timed-out wait
    return flmm_context_check(s->ctx, stream);
}
