// noalloc.cu -- Jacobi-preconditioned CG on a caller's CSR matrix that
// allocates no device memory.
//
// Callers that cannot allocate on the device (a render loop that must not
// stall on cudaMalloc/cudaFree, a host framework that owns the whole memory
// pool, code that must not fail with out-of-memory half way through a frame)
// pass the matrix, the right-hand side and the solution vector; the CG work
// vectors and reduction partials live in one static device array below.
//
// Limits: the work vectors r, p, q and D^-1 take 4 * n * sizeof(real) bytes
// of a 16 MiB region, so n <= 1,048,576 unknowns in FP32 and <= 524,288 in
// FP64; the state and block partials use a further 64 KiB.  Every GPU that
// loads the library holds these 16 MiB + 64 KiB until the process exits.
//
// The array is shared by all calls on a device and keeps the last call's
// contents: each call clears the loop state before use, and calls that
// overlap on the GPU (other streams, other host threads) race on it.
//
// Outcome: FEA_STATUS_* bits of the solve (breakdown, non-finite values, no
// convergence within max_iterations); breakdown and non-finite values also
// make the call return FEA_ERR_SOLVE, since x is then no solution.  The host
// reads the loop condition once per kNaItersPerCheck iterations: the kernels
// of iterations past the end return at once.
//
// Inner products and the initial residual accumulate in the solvers' exact
// accumulators (float-float pairs in FP32), block and grid totals included.
#include <cmath>
#include <mutex>

#include "cg_device.cuh"

namespace fea {
namespace {

constexpr int kNaMaxBlocks = 1024;
constexpr size_t kNaVecBytes = (size_t)16 << 20;
constexpr size_t kNaHeadBytes = (size_t)64 << 10;
constexpr int kNaMaxDevices = 64;

constexpr int kNaItersPerCheck = 8;

struct NaState {
    double bb, rr, rz, pq, thr, alpha, beta;
    int active, iter, max_iter, cont, zero_rhs;
    unsigned int flags;  // FEA_STATUS_*
    unsigned int ticket[4];
};
constexpr size_t kNaPartOffset = 256;
static_assert(sizeof(NaState) <= kNaPartOffset, "state header");
static_assert(kNaPartOffset + 3 * kNaMaxBlocks * sizeof(double) <= kNaHeadBytes, "partials");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaHeadBytes + kNaVecBytes];

std::mutex g_na_mutex;
void* g_na_ptr[kNaMaxDevices] = {};

template <typename R>
struct NaArgs {
    int n;
    const int32_t* rp;
    const int32_t* col;
    const R* val;
    const R* b;
    R* x;
    NaState* st;
    double* part;
    R *r, *p, *q, *dinv;
};

template <int NV, typename R>
__device__ __forceinline__ bool na_reduce(Acc<R> (&acc)[NV], double* part, unsigned int* ticket, double (&out)[NV]) {
    __shared__ typename Acc<R>::Packed sm[32 * NV];
    Acc<R> blk[NV], tot[NV];
    block_totals<NV, R>(acc, sm, blk);
    const bool last = grid_commit<NV, R>(blk, part, kNaMaxBlocks, ticket, sm, tot);
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = tot[k].value();
    return last;
}

// r = b - A x, D^-1, p = D^-1 r and the set-up scalars.
template <typename R>
__global__ void __launch_bounds__(kBlock) k_na_init(NaArgs<R> a, double tol, int max_iter) {
    Acc<R> acc[3];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        Acc<R> t;
        R d = 0;
        for (int32_t e = a.rp[i]; e < a.rp[i + 1]; e++) {
            const int32_t c = a.col[e];
            t.add_prod(-a.val[e], a.x[c]);
            if (c == i) d += a.val[e];
        }
        const R bi = a.b[i];
        t.add(bi);
        const R ri = t.rounded();
        const R di = d != (R)0 ? (R)1 / d : (R)1;
        a.r[i] = ri;
        a.dinv[i] = di;
        a.p[i] = di * ri;
        acc[0].add_prod(bi, bi);
        acc[1].add_prod(ri, ri);
        acc[2].add_prod(ri, di * ri);
    }
    double tot[3];
    if (na_reduce<3>(acc, a.part, &a.st->ticket[0], tot) && threadIdx.x == 0) {
        NaState* st = a.st;
        const double tiny = sizeof(R) == 4 ? 1.1754943508222875e-38 : 2.2250738585072014e-308;
        st->bb = tot[0];
        st->rr = tot[1];
        st->rz = tot[2];
        st->thr = fmax(tol * tol * tot[0], tiny);
        st->iter = 0;
        st->max_iter = max_iter;
        if (!isfinite(tot[0]) || !isfinite(tot[1]) || !isfinite(tot[2])) {  // NaN or Inf in A, b or x
            st->flags |= FEA_STATUS_NONFINITE;
            st->zero_rhs = 0;
            st->active = 0;
        } else {
            st->zero_rhs = !(tot[0] > 0.0);  // Eigen's early exit: x = 0
            st->active = !st->zero_rhs && tot[1] >= st->thr;
        }
        st->cont = st->active;
    }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_na_spmv(NaArgs<R> a) {
    if (!a.st->active) return;
    Acc<R> acc[1];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        R s = 0;
        for (int32_t e = a.rp[i]; e < a.rp[i + 1]; e++) s = fmar(a.val[e], a.p[a.col[e]], s);
        a.q[i] = s;
        acc[0].add_prod(a.p[i], s);
    }
    double tot[1];
    if (na_reduce<1>(acc, a.part, &a.st->ticket[1], tot) && threadIdx.x == 0) {
        NaState* st = a.st;
        st->pq = tot[0];
        const double al = st->rz / tot[0];
        if (!(tot[0] > 0.0) || !isfinite(al)) {  // p.Ap <= 0: A is not SPD (or non-finite)
            st->flags |= isfinite(tot[0]) ? FEA_STATUS_BREAKDOWN : FEA_STATUS_BREAKDOWN | FEA_STATUS_NONFINITE;
            st->active = 0;
            st->cont = 0;
        } else {
            st->alpha = al;
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_na_update(NaArgs<R> a) {
    if (!a.st->active) return;
    const R alpha = (R)a.st->alpha;
    Acc<R> acc[2];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        a.x[i] = fmar(alpha, a.p[i], a.x[i]);
        const R ri = fmar(-alpha, a.q[i], a.r[i]);
        a.r[i] = ri;
        acc[0].add_prod(ri, a.dinv[i] * ri);
        acc[1].add_prod(ri, ri);
    }
    double tot[2];
    if (na_reduce<2>(acc, a.part, &a.st->ticket[2], tot) && threadIdx.x == 0) {
        NaState* st = a.st;
        st->iter += 1;
        st->rr = tot[1];
        if (!isfinite(tot[0]) || !isfinite(tot[1])) {
            st->flags |= FEA_STATUS_NONFINITE;
            st->active = 0;
            st->cont = 0;
        } else if (tot[1] < st->thr) {  // converged
            st->active = 0;
            st->cont = 0;
        } else {
            st->beta = tot[0] / st->rz;
            st->rz = tot[0];
            if (!isfinite(st->beta)) st->flags |= FEA_STATUS_BREAKDOWN;
            st->cont = isfinite(st->beta) && st->iter < st->max_iter;
            if (isfinite(st->beta) && !st->cont) st->flags |= FEA_STATUS_NOT_CONVERGED;
            st->active = st->cont;
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_na_dir(NaArgs<R> a) {
    if (!a.st->active) return;
    const R beta = (R)a.st->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x)
        a.p[i] = fmar(beta, a.p[i], a.dinv[i] * a.r[i]);
}

// Eigen's early exit: a zero right-hand side gives x = 0.
template <typename R>
__global__ void k_na_zero(NaArgs<R> a) {
    if (!a.st->zero_rhs) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) a.x[i] = 0;
}

// Device address of the static scratch on the current device, looked up once
// per device (with that device current).
int na_scratch(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(FEA_ERR_NO_DEVICE, cudaGetErrorString(e));
    if (dev < 0 || dev >= kNaMaxDevices) return fail(FEA_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error("cudaGetSymbolAddress of the static scratch failed: %s", cudaGetErrorString(e));
            return FEA_ERR_CUDA;
        }
        g_na_ptr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_na_ptr[dev]);
    return FEA_OK;
}

template <typename R>
int na_solve(int64_t n, const int32_t* rp, const int32_t* col, const void* val, const void* b, void* x,
             double tol, int max_iter, cudaStream_t st, int* iterations, double* rel_res, unsigned int* flags) {
    unsigned char* base = nullptr;
    int rc = na_scratch(&base);
    if (rc != FEA_OK) return rc;
    NaArgs<R> a{};
    a.n = (int)n;
    a.rp = rp;
    a.col = col;
    a.val = static_cast<const R*>(val);
    a.b = static_cast<const R*>(b);
    a.x = static_cast<R*>(x);
    a.st = reinterpret_cast<NaState*>(base);
    a.part = reinterpret_cast<double*>(base + kNaPartOffset);
    R* vec = reinterpret_cast<R*>(base + kNaHeadBytes);
    a.r = vec;
    a.p = vec + n;
    a.q = vec + 2 * n;
    a.dinv = vec + 3 * n;
    if (!(tol > 0.0)) tol = sizeof(R) == 4 ? 1.1920928955078125e-07 : 1e-10;
    if (max_iter <= 0) max_iter = (int)(2 * n < 0x7fffffff ? 2 * n : 0x7fffffff);
    int grid = (int)ceil_div(n, kBlock);
    if (grid > kNaMaxBlocks) grid = kNaMaxBlocks;
    if (grid < 1) grid = 1;
    // the loop state and reduction tickets must start at zero on every call
    cudaError_t e = cudaMemsetAsync(a.st, 0, sizeof(NaState), st);
    if (e != cudaSuccess) return fail(FEA_ERR_CUDA, cudaGetErrorString(e));
    k_na_init<R><<<grid, kBlock, 0, st>>>(a, tol, max_iter);
    int64_t it = 0;
    for (;;) {  // the loop condition is read once per kNaItersPerCheck iterations
        int cont = 0;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&cont, &a.st->cont, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return fail(FEA_ERR_CUDA, cudaGetErrorString(e));
        if (!cont || it > max_iter) break;
        for (int k = 0; k < kNaItersPerCheck; k++) {  // iterations past the end return at once
            k_na_spmv<R><<<grid, kBlock, 0, st>>>(a);
            k_na_update<R><<<grid, kBlock, 0, st>>>(a);
            k_na_dir<R><<<grid, kBlock, 0, st>>>(a);
        }
        it += kNaItersPerCheck;
    }
    k_na_zero<R><<<grid, kBlock, 0, st>>>(a);
    NaState h{};
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, a.st, sizeof(NaState), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(FEA_ERR_CUDA, cudaGetErrorString(e));
    if (iterations) *iterations = h.iter;
    if (rel_res) *rel_res = h.bb > 0.0 && isfinite(h.rr) ? sqrt(h.rr / h.bb) : (h.flags ? NAN : 0.0);
    if (flags) *flags = h.flags;
    if (h.flags & (FEA_STATUS_BREAKDOWN | FEA_STATUS_NONFINITE)) {
        set_error("solve failed: %s", (h.flags & FEA_STATUS_NONFINITE) ? "non-finite values in A, b, x or the iterates"
                                                                     : "breakdown (p.Ap <= 0: the matrix is not SPD)");
        return FEA_ERR_SOLVE;
    }
    return FEA_OK;
}

}  // namespace
}  // namespace fea

extern "C" int fea_pcg_solve_csr_noalloc(int64_t n, const int32_t* row_ptr, const int32_t* col, const void* values,
                                         const void* b, void* x, int precision, double tolerance,
                                         int max_iterations, void* stream, int* iterations,
                                         double* rel_residual, unsigned int* status_flags) {
    using namespace fea;
    if (precision != FEA_FP32 && precision != FEA_FP64) return fail(FEA_ERR_INVALID_ARGUMENT, "bad precision");
    const size_t rsz = precision == FEA_FP64 ? sizeof(double) : sizeof(float);
    const int64_t max_n = (int64_t)(kNaVecBytes / (4 * rsz));
    if (n < 0 || n > max_n) {
        set_error("n = %lld exceeds the no-allocation limit of %lld unknowns (%s; 16 MiB of static scratch)",
                  (long long)n, (long long)max_n, precision == FEA_FP64 ? "FP64" : "FP32");
        return FEA_ERR_TOO_LARGE;
    }
    if (n == 0) {
        if (iterations) *iterations = 0;
        if (rel_residual) *rel_residual = 0.0;
        if (status_flags) *status_flags = 0u;
        return FEA_OK;
    }
    if (!row_ptr || !col || !values || !b || !x) return fail(FEA_ERR_INVALID_ARGUMENT, "null array");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (precision == FEA_FP64)
        return na_solve<double>(n, row_ptr, col, values, b, x, tolerance, max_iterations, st, iterations,
                                rel_residual, status_flags);
    return na_solve<float>(n, row_ptr, col, values, b, x, tolerance, max_iterations, st, iterations, rel_residual,
                           status_flags);
}
