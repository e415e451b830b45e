// Learned e-value tail: a 256 -> 128 -> 64 -> 3 MLP (FP32) that maps a
// spectrum's hyperscore histogram to the tail-fit line of expeRT
// (slope, intercept, first regression bin; expeRT.cpp:646-704), trained and
// run with the kernels below. The expeRT fit (k_tailfit) is the training
// target, the fallback whenever the predicted line misfits the spectrum's own
// survival curve, and the judge of the e-value error.
//
// Input features (fixed, not learned): bins 0..254 of the histogram and the
// sum of bins >= 255 in bin 255, turned into the log10 survival curve
// log10(1 - cumsum/cpsms) (clamped at -7) the regression is fitted to; bins at
// and above the top hit's bin (excluded by expeRT, expeRT.cpp:590) repeat the
// last value below it.
#include <cmath>
#include <cstring>
#include <vector>

#include "hc_internal.h"

struct hc_mlp
{
    hc_ctx *ctx = nullptr;
    float *d_params = nullptr;  // W1 b1 W2 b2 W3 b3
    float *d_grads = nullptr;
    float *d_m = nullptr, *d_v = nullptr;
    float *d_act = nullptr;     // activations for one minibatch: h1 | h2 | out | dout | dh2 | dh1
    size_t act_cap = 0;
    float *d_loss = nullptr;
    int step = 0;
};

namespace hc {
namespace {

constexpr int kIn = 256, kH1 = 128, kH2 = 64, kOut = 3;
constexpr size_t kOffW1 = 0, kOffB1 = kOffW1 + kIn * kH1, kOffW2 = kOffB1 + kH1, kOffB2 = kOffW2 + kH1 * kH2,
                 kOffW3 = kOffB2 + kH2, kOffB3 = kOffW3 + kH2 * kOut, kParams = kOffB3 + kOut;
// target scaling: slope x 10, intercept / 4, first bin / 50
__host__ __device__ constexpr float tscale(int j) { return j == 0 ? 10.0f : (j == 1 ? 0.25f : 0.02f); }

// ---- features -------------------------------------------------------------
__global__ void k_features(const uint32_t *__restrict__ hist, const hc_result *__restrict__ res, uint32_t n,
                           float *__restrict__ X)
{
    const uint32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= n) return;
    const uint32_t *h = hist + (size_t)s * HC_HIST_BINS;
    const hc_result r = res[s];
    const float cps = (float)(r.cpsms > 0 ? r.cpsms : 1);
    int hyp = (int)__dadd_rn((double)__fmul_rn(r.hyperscore, 10.0f), 0.5);
    if (hyp > kIn) hyp = kIn;
    // fold bins >= 255 into 255
    uint32_t tailsum = 0;
    for (int b = 255 + lane; b < HC_HIST_BINS; b += 32) tailsum += h[b];
    tailsum = __reduce_add_sync(0xFFFFFFFFu, tailsum);
    uint32_t carry = 0;
    float *x = X + (size_t)s * kIn;
    for (int b0 = 0; b0 < kIn; b0 += 32)
    {
        const int b = b0 + lane;
        uint32_t v = (b < 255) ? h[b] : tailsum;
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
            if (lane >= o) v += t;
        }
        const float sv = 1.0f - (float)(carry + v) / cps;
        x[b] = log10f(fmaxf(sv, 1e-7f));
        carry += __shfl_sync(0xFFFFFFFFu, v, 31);
    }
    __syncwarp();
    // bins at/after the top hit's bin repeat the last value below it
    const float last = hyp > 0 ? x[hyp - 1] : 0.0f;
    __syncwarp();
    for (int b = hyp + lane; b < kIn; b += 32) x[b] = last;
}

__global__ void k_targets(const hc_result *__restrict__ res, const int32_t *__restrict__ fitstart, uint32_t n,
                          float *__restrict__ Y)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const hc_result r = res[s];
    Y[s * kOut + 0] = (float)((double)r.mu / 1e6);
    Y[s * kOut + 1] = (float)((double)r.beta / 1e6);
    Y[s * kOut + 2] = (float)(fitstart[s] < 0 ? 0 : fitstart[s]);
}

// ---- dense layers (row-major: Y[n,N] = X[n,K] W[K,N] + b) -----------------
constexpr int TB = 32;

__global__ void k_linear(const float *__restrict__ X, const float *__restrict__ W, const float *__restrict__ b,
                         float *__restrict__ Y, int n, int K, int N, int relu)
{
    __shared__ float xs[TB][TB + 1], ws[TB][TB + 1];
    const int r = blockIdx.y * TB + threadIdx.y, c = blockIdx.x * TB + threadIdx.x;
    float acc = 0.0f;
    for (int k0 = 0; k0 < K; k0 += TB)
    {
        xs[threadIdx.y][threadIdx.x] = (r < n && k0 + threadIdx.x < K) ? X[(size_t)r * K + k0 + threadIdx.x] : 0.0f;
        ws[threadIdx.y][threadIdx.x] = (k0 + threadIdx.y < K && c < N) ? W[(size_t)(k0 + threadIdx.y) * N + c] : 0.0f;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < TB; k++) acc += xs[threadIdx.y][k] * ws[k][threadIdx.x];
        __syncthreads();
    }
    if (r < n && c < N)
    {
        float v = acc + b[c];
        Y[(size_t)r * N + c] = relu ? fmaxf(v, 0.0f) : v;
    }
}

// dX[n,K] = (dY[n,N] W^T) * (X > 0)   (X = the layer input after its ReLU)
__global__ void k_linear_bwd_x(const float *__restrict__ dY, const float *__restrict__ W,
                               const float *__restrict__ Xin, float *__restrict__ dX, int n, int K, int N)
{
    __shared__ float ds[TB][TB + 1], ws[TB][TB + 1];
    const int r = blockIdx.y * TB + threadIdx.y, c = blockIdx.x * TB + threadIdx.x;  // c indexes K
    float acc = 0.0f;
    for (int j0 = 0; j0 < N; j0 += TB)
    {
        ds[threadIdx.y][threadIdx.x] = (r < n && j0 + threadIdx.x < N) ? dY[(size_t)r * N + j0 + threadIdx.x] : 0.0f;
        const int wc = blockIdx.x * TB + threadIdx.y;  // row of W (a K index)
        ws[threadIdx.y][threadIdx.x] = (wc < K && j0 + threadIdx.x < N) ? W[(size_t)wc * N + j0 + threadIdx.x] : 0.0f;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < TB; j++) acc += ds[threadIdx.y][j] * ws[threadIdx.x][j];
        __syncthreads();
    }
    if (r < n && c < K) dX[(size_t)r * K + c] = Xin[(size_t)r * K + c] > 0.0f ? acc : 0.0f;
}

// dW[K,N] = X^T dY, db[N] = sum_rows dY   (one thread per output, rows tiled)
__global__ void k_linear_bwd_w(const float *__restrict__ X, const float *__restrict__ dY, float *__restrict__ dW,
                               float *__restrict__ db, int n, int K, int N)
{
    __shared__ float xs[TB][TB + 1], ds[TB][TB + 1];
    const int k = blockIdx.y * TB + threadIdx.y, c = blockIdx.x * TB + threadIdx.x;
    float acc = 0.0f, accb = 0.0f;
    for (int r0 = 0; r0 < n; r0 += TB)
    {
        const int rx = r0 + threadIdx.x;  // row index for the transposed X tile
        xs[threadIdx.y][threadIdx.x] = (rx < n && blockIdx.y * TB + threadIdx.y < K)
                                           ? X[(size_t)rx * K + blockIdx.y * TB + threadIdx.y] : 0.0f;
        ds[threadIdx.y][threadIdx.x] = (r0 + threadIdx.y < n && c < N) ? dY[(size_t)(r0 + threadIdx.y) * N + c] : 0.0f;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < TB; r++)
        {
            acc += xs[threadIdx.y][r] * ds[r][threadIdx.x];
            accb += ds[r][threadIdx.x];
        }
        __syncthreads();
    }
    if (k < K && c < N) dW[(size_t)k * N + c] = acc;
    if (blockIdx.y == 0 && threadIdx.y == 0 && c < N) db[c] = accb;
}

// MSE on scaled targets: dOut = 2 (out - t) / (n * 3); loss accumulated
__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ Y, int n, float *__restrict__ dOut,
                      float *__restrict__ loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < n * kOut)
    {
        const float t = Y[i] * tscale(i % kOut);
        const float d = out[i] - t;
        dOut[i] = 2.0f * d / (float)(n * kOut);
        l = d * d / (float)(n * kOut);
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xFFFFFFFFu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       size_t n, float lr, float b1t, float b2t)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = 0.9f * m[i] + 0.1f * gi;
    const float vi = 0.999f * v[i] + 0.001f * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / (1.0f - b1t)) / (sqrtf(vi / (1.0f - b2t)) + 1e-8f);
}

// Learned e-value, one warp per spectrum (res holds the expeRT fit, which
// stays the fallback). The survival curve is the feature vector itself
// (log10 survival per bin) over the bins the reference fits, [stt1, end1]
// (expeRT.cpp:590-598). The regression window's upper end is expeRT's rule
// (last point above 87 % of the curve's drop, expeRT.cpp:662-676); its start
// is the network's third output in place of expeRT's 22 % rule (646-661). The
// line is the least-squares fit of the curve over that window; its RMS
// residual there (log10 units) must be within `thresh` (a straight tail over
// the chosen window), else the spectrum keeps its expeRT e-value.
// mode 0: network window; mode 1: window from the curve's first bin (the
// same refit without the network, for comparison); mode 2: mode 0, and the
// network's predicted line (expeRT's slope and intercept) must also agree
// with the refitted line at the top hit within `thresh`.
__global__ void k_learned_evalue(const float *__restrict__ X, const float *__restrict__ out, hc_result *__restrict__ res,
                                 uint32_t n, float thresh, uint32_t min_cpsm, double expect_max, int mode,
                                 float *__restrict__ learned_log10e, uint32_t *__restrict__ nfallback)
{
    const uint32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= n) return;
    hc_result r = res[s];
    if (r.cpsms < min_cpsm || r.cpsms == 0)
    {
        if (lane == 0) learned_log10e[s] = NAN;
        return;
    }
    const float *x = X + (size_t)s * kIn;
    const int hyp = r.maxhyp, stt1 = r.minhyp;
    int end1 = r.nexthyp;
    if (stt1 == end1) end1 += 1;
    const int nb = end1 - stt1 + 1;
    bool fb = hyp >= kIn || end1 >= kIn || stt1 < 0 || nb < 4;
    int first = 0, last = 0;
    if (!fb)
    {
        // upper end: the last point at or above y0 + 0.87 (y_{n-1} - y0)
        const float y0 = x[stt1], t2 = y0 + 0.87f * (x[end1] - y0);
        int m2 = nb - 1;
        for (int q0 = nb - 1; q0 >= 0; q0 -= 32)
        {
            const int q = q0 - lane;
            const uint32_t b = __ballot_sync(0xFFFFFFFFu, q >= 0 && x[stt1 + q] >= t2);
            if (b) { m2 = q0 - (__ffs(b) - 1); break; }
        }
        last = stt1 + m2;
        if (mode != 1) first = (int)lrintf(out[s * kOut + 2] / tscale(2));
        else first = stt1;
        first = max(stt1, min(first, last - 1));
        fb = last - first < 1;
    }
    float slope = 0.0f, icpt = 0.0f, resid = 1e30f;
    if (!fb)
    {
        const int m = last - first + 1;
        const float xbar = 0.5f * (float)(first + last);
        float sy = 0.0f;
        for (int i = lane; i < m; i += 32) sy += x[first + i];
        for (int o = 16; o > 0; o >>= 1) sy += __shfl_xor_sync(0xFFFFFFFFu, sy, o);
        const float ybar = sy / (float)m;
        float top = 0.0f, bot = 0.0f;
        for (int i = lane; i < m; i += 32)
        {
            const float dx = (float)(first + i) - xbar, y = x[first + i];
            top += dx * (y - ybar);
            bot += dx * dx;
        }
        for (int o = 16; o > 0; o >>= 1)
        {
            top += __shfl_xor_sync(0xFFFFFFFFu, top, o);
            bot += __shfl_xor_sync(0xFFFFFFFFu, bot, o);
        }
        slope = top / bot;
        icpt = ybar - slope * xbar;
        float se = 0.0f;
        for (int i = lane; i < m; i += 32)
        {
            const float d = slope * (float)(first + i) + icpt - x[first + i];
            se += d * d;
        }
        for (int o = 16; o > 0; o >>= 1) se += __shfl_xor_sync(0xFFFFFFFFu, se, o);
        resid = mode != 1 ? sqrtf(se / (float)m) : 0.0f;
    }
    if (lane != 0) return;
    // mode 2: the refitted line and the network's predicted line (expeRT's
    // slope and intercept) at the top hit's hyperscore bin
    const float agree = mode == 2 && !fb
                            ? fabsf((slope - out[s * kOut + 0] / tscale(0)) * (float)hyp +
                                    (icpt - out[s * kOut + 1] / tscale(1)))
                            : 0.0f;
    if (fb || !(resid <= thresh) || !(agree <= thresh))
    {
        learned_log10e[s] = NAN;
        atomicAdd(nfallback, 1u);  // keep the expeRT value already in res
        return;
    }
    const double lg = (double)slope * (double)hyp + (double)icpt + log10((double)r.cpsms);
    learned_log10e[s] = (float)lg;
    r.evalue = pow(10.0, lg);
    r.reported = r.evalue < expect_max ? 1u : 0u;
    r.flags |= HC_FLAG_LEARNED;
    res[s] = r;
}

}  // namespace

static int mlp_forward(hc_mlp *m, const float *X, uint32_t n, float *h1, float *h2, float *out, cudaStream_t st)
{
    const float *P = m->d_params;
    dim3 blk(TB, TB);
    k_linear<<<dim3((kH1 + TB - 1) / TB, (n + TB - 1) / TB), blk, 0, st>>>(X, P + kOffW1, P + kOffB1, h1, n, kIn, kH1, 1);
    k_linear<<<dim3((kH2 + TB - 1) / TB, (n + TB - 1) / TB), blk, 0, st>>>(h1, P + kOffW2, P + kOffB2, h2, n, kH1, kH2, 1);
    k_linear<<<dim3((kOut + TB - 1) / TB, (n + TB - 1) / TB), blk, 0, st>>>(h2, P + kOffW3, P + kOffB3, out, n, kH2, kOut, 0);
    HC_CUDA(m->ctx, cudaGetLastError());
    return HC_SUCCESS;
}

static int ensure_act(hc_mlp *m, uint32_t n)
{
    const size_t need = (size_t)n * (kH1 + kH2 + kOut) * 2;
    if (m->act_cap >= need) return HC_SUCCESS;
    cudaFree(m->d_act);
    m->d_act = nullptr;
    m->act_cap = 0;
    HC_CUDA(m->ctx, cudaMalloc((void **)&m->d_act, sizeof(float) * need));
    m->act_cap = need;
    return HC_SUCCESS;
}

// forward + backward of one minibatch; gradients land in d_grads
static int mlp_fwd_bwd(hc_mlp *m, const float *X, const float *Y, uint32_t n, cudaStream_t st)
{
    int rc = ensure_act(m, n);
    if (rc) return rc;
    float *h1 = m->d_act, *h2 = h1 + (size_t)n * kH1, *out = h2 + (size_t)n * kH2;
    float *dout = out + (size_t)n * kOut, *dh2 = dout + (size_t)n * kOut, *dh1 = dh2 + (size_t)n * kH2;
    if ((rc = mlp_forward(m, X, n, h1, h2, out, st))) return rc;
    const float *P = m->d_params;
    float *G = m->d_grads;
    k_mse<<<(n * kOut + 255) / 256, 256, 0, st>>>(out, Y, (int)n, dout, m->d_loss);
    dim3 blk(TB, TB);
    k_linear_bwd_w<<<dim3((kOut + TB - 1) / TB, (kH2 + TB - 1) / TB), blk, 0, st>>>(h2, dout, G + kOffW3, G + kOffB3, n, kH2, kOut);
    k_linear_bwd_x<<<dim3((kH2 + TB - 1) / TB, (n + TB - 1) / TB), blk, 0, st>>>(dout, P + kOffW3, h2, dh2, n, kH2, kOut);
    k_linear_bwd_w<<<dim3((kH2 + TB - 1) / TB, (kH1 + TB - 1) / TB), blk, 0, st>>>(h1, dh2, G + kOffW2, G + kOffB2, n, kH1, kH2);
    k_linear_bwd_x<<<dim3((kH1 + TB - 1) / TB, (n + TB - 1) / TB), blk, 0, st>>>(dh2, P + kOffW2, h1, dh1, n, kH1, kH2);
    k_linear_bwd_w<<<dim3((kH1 + TB - 1) / TB, (kIn + TB - 1) / TB), blk, 0, st>>>(X, dh1, G + kOffW1, G + kOffB1, n, kIn, kH1);
    HC_CUDA(m->ctx, cudaGetLastError());
    return HC_SUCCESS;
}

}  // namespace hc

using namespace hc;

extern "C" {

int hc_mlp_create(hc_ctx *ctx, uint64_t seed, hc_mlp **out)
{
    if (!ctx || !out) return HC_ERR_INVLD_PTR;
    cudaSetDevice(ctx->device);
    hc_mlp *m = new hc_mlp();
    m->ctx = ctx;
    std::vector<float> h(kParams, 0.0f);
    // He-uniform initialisation from a splitmix64 stream
    uint64_t x = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        x += 0x9E3779B97F4A7C15ull;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return (double)((z ^ (z >> 31)) >> 11) / 9007199254740992.0;
    };
    auto fill = [&](size_t off, int fan_in, size_t cnt) {
        const double lim = std::sqrt(6.0 / fan_in);
        for (size_t i = 0; i < cnt; i++) h[off + i] = (float)((2.0 * next() - 1.0) * lim);
    };
    fill(kOffW1, kIn, (size_t)kIn * kH1);
    fill(kOffW2, kH1, (size_t)kH1 * kH2);
    fill(kOffW3, kH2, (size_t)kH2 * kOut);
    if (cudaMalloc((void **)&m->d_params, 4 * kParams) != cudaSuccess ||
        cudaMalloc((void **)&m->d_grads, 4 * kParams) != cudaSuccess ||
        cudaMalloc((void **)&m->d_m, 4 * kParams) != cudaSuccess ||
        cudaMalloc((void **)&m->d_v, 4 * kParams) != cudaSuccess ||
        cudaMalloc((void **)&m->d_loss, 16) != cudaSuccess)
    {
        delete m;
        return HC_ERR_BAD_MEM_ALLOC;
    }
    cudaMemcpy(m->d_params, h.data(), 4 * kParams, cudaMemcpyHostToDevice);
    cudaMemset(m->d_m, 0, 4 * kParams);
    cudaMemset(m->d_v, 0, 4 * kParams);
    *out = m;
    return HC_SUCCESS;
}

int hc_mlp_destroy(hc_mlp *m)
{
    if (!m) return HC_ERR_INVLD_PTR;
    cudaFree(m->d_params);
    cudaFree(m->d_grads);
    cudaFree(m->d_m);
    cudaFree(m->d_v);
    cudaFree(m->d_act);
    cudaFree(m->d_loss);
    delete m;
    return HC_SUCCESS;
}

int hc_mlp_num_params(void) { return (int)kParams; }

int hc_mlp_get_params(hc_mlp *m, float *host)
{
    if (!m || !host) return HC_ERR_INVLD_PTR;
    HC_CUDA(m->ctx, cudaMemcpy(host, m->d_params, 4 * kParams, cudaMemcpyDeviceToHost));
    return HC_SUCCESS;
}

int hc_mlp_set_params(hc_mlp *m, const float *host)
{
    if (!m || !host) return HC_ERR_INVLD_PTR;
    HC_CUDA(m->ctx, cudaMemcpy(m->d_params, host, 4 * kParams, cudaMemcpyHostToDevice));
    return HC_SUCCESS;
}

int hc_mlp_features(hc_ctx *ctx, const uint32_t *d_hist, const hc_result *d_res, uint32_t n, float *d_X, void *stream)
{
    if (!ctx || (n && (!d_hist || !d_res || !d_X))) return HC_ERR_INVLD_PTR;
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    if (n) k_features<<<(n + 3) / 4, 128, 0, st>>>(d_hist, d_res, n, d_X);
    HC_CUDA(ctx, cudaGetLastError());
    return HC_SUCCESS;
}

int hc_mlp_targets(hc_ctx *ctx, const hc_result *d_res, uint32_t n, float *d_Y, void *stream)
{
    if (!ctx || (n && (!d_res || !d_Y))) return HC_ERR_INVLD_PTR;
    if (n > ctx->qs.fit_cap) return set_error(ctx, HC_ERR_INVLD_SIZE, "targets need the last query's fit starts");
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    if (n) k_targets<<<(n + 255) / 256, 256, 0, st>>>(d_res, ctx->qs.d_fitstart, n, d_Y);
    HC_CUDA(ctx, cudaGetLastError());
    return HC_SUCCESS;
}

int hc_mlp_forward(hc_mlp *m, const float *d_X, uint32_t n, float *d_out, void *stream)
{
    if (!m || (n && (!d_X || !d_out))) return HC_ERR_INVLD_PTR;
    cudaStream_t st = stream ? (cudaStream_t)stream : m->ctx->stream;
    int rc = ensure_act(m, n);
    if (rc) return rc;
    float *h1 = m->d_act, *h2 = h1 + (size_t)n * kH1;
    return mlp_forward(m, d_X, n, h1, h2, d_out, st);
}

int hc_mlp_gradients(hc_mlp *m, const float *d_X, const float *d_Y, uint32_t n, float *host_grads, float *loss)
{
    if (!m || !d_X || !d_Y) return HC_ERR_INVLD_PTR;
    cudaStream_t st = m->ctx->stream;
    HC_CUDA(m->ctx, cudaMemsetAsync(m->d_loss, 0, 4, st));
    int rc = mlp_fwd_bwd(m, d_X, d_Y, n, st);
    if (rc) return rc;
    if (host_grads) HC_CUDA(m->ctx, cudaMemcpyAsync(host_grads, m->d_grads, 4 * kParams, cudaMemcpyDeviceToHost, st));
    if (loss) HC_CUDA(m->ctx, cudaMemcpyAsync(loss, m->d_loss, 4, cudaMemcpyDeviceToHost, st));
    HC_CUDA(m->ctx, cudaStreamSynchronize(st));
    return HC_SUCCESS;
}

int hc_mlp_train(hc_mlp *m, const float *d_X, const float *d_Y, uint32_t n, uint32_t batch, uint32_t epochs,
                 float lr, float *final_loss)
{
    if (!m || !d_X || !d_Y || batch == 0) return HC_ERR_INVLD_PTR;
    cudaStream_t st = m->ctx->stream;
    float loss = 0.0f;
    for (uint32_t ep = 0; ep < epochs; ep++)
    {
        HC_CUDA(m->ctx, cudaMemsetAsync(m->d_loss, 0, 4, st));
        uint32_t nb = 0;
        for (uint32_t s0 = 0; s0 < n; s0 += batch)
        {
            const uint32_t b = std::min(batch, n - s0);
            int rc = mlp_fwd_bwd(m, d_X + (size_t)s0 * kIn, d_Y + (size_t)s0 * kOut, b, st);
            if (rc) return rc;
            m->step++;
            const float b1t = std::pow(0.9f, (float)m->step), b2t = std::pow(0.999f, (float)m->step);
            k_adam<<<(unsigned)((kParams + 255) / 256), 256, 0, st>>>(m->d_params, m->d_grads, m->d_m, m->d_v, kParams,
                                                                       lr, b1t, b2t);
            nb++;
        }
        HC_CUDA(m->ctx, cudaMemcpyAsync(&loss, m->d_loss, 4, cudaMemcpyDeviceToHost, st));
        HC_CUDA(m->ctx, cudaStreamSynchronize(st));
        loss /= (float)(nb ? nb : 1);
    }
    if (final_loss) *final_loss = loss;
    return HC_SUCCESS;
}

int hc_mlp_evalues(hc_mlp *m, const float *d_X, hc_result *d_res, uint32_t n, float thresh, float *d_learned_log10e,
                   uint32_t *d_nfallback, float *d_out_scratch, void *stream)
{
    return hc_mlp_evalues_mode(m, d_X, d_res, n, thresh, 0, d_learned_log10e, d_nfallback, d_out_scratch, stream);
}

int hc_mlp_evalues_mode(hc_mlp *m, const float *d_X, hc_result *d_res, uint32_t n, float thresh, int mode,
                        float *d_learned_log10e, uint32_t *d_nfallback, float *d_out_scratch, void *stream)
{
    if (mode < 0 || mode > 2) return HC_ERR_INVLD_PARAM;
    if (!m || (n && (!d_X || !d_res || !d_learned_log10e || !d_nfallback || !d_out_scratch))) return HC_ERR_INVLD_PTR;
    cudaStream_t st = stream ? (cudaStream_t)stream : m->ctx->stream;
    int rc = hc_mlp_forward(m, d_X, n, d_out_scratch, st);
    if (rc) return rc;
    if (n)
        k_learned_evalue<<<(n + 3) / 4, 128, 0, st>>>(d_X, d_out_scratch, d_res, n, thresh, m->ctx->p.min_cpsm,
                                                      m->ctx->p.expect_max, mode, d_learned_log10e, d_nfallback);
    HC_CUDA(m->ctx, cudaGetLastError());
    return HC_SUCCESS;
}

}  // extern "C"
