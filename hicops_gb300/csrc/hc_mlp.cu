// Learned e-value tail: a 256 -> 128 -> 64 -> 4 MLP (FP32) that maps a
// spectrum's hyperscore histogram to the tail of its survival function, in
// place of the per-spectrum regression fit of expeRT (expeRT::ModelTailFit,
// expeRT.cpp:572-718), which stays the fallback and the yardstick.
//
// Outputs: the tail line (slope, intercept), the first bin of the regression
// window (expeRT picks it by searching the curve for its 22 % point,
// expeRT.cpp:646-661) and the RMS residual of the line over the window.
//
// Input features (fixed, not learned): bins 0..254 of the histogram and the
// sum of bins >= 255 in bin 255, turned into the log10 survival curve
// log10(1 - cumsum/cpsms) (clamped at -7); bins at and above the top hit's bin
// (excluded by expeRT, expeRT.cpp:590) repeat the last value below it.
//
// The learned e-value (k_learned_tail). A spectrum whose predicted residual
// exceeds the gate (0.1, log10 units) goes to expeRT at once. Otherwise its
// survival curve over expeRT's bins [stt1, end1] is formed in FP32 from the
// full histogram, and the network's first bin is confirmed on it: the curve
// is monotone, so the first bin is expeRT's exactly when the point after it
// is the first at or below the 22 % level, a test of two points; the kernel
// tests the predicted bin and its neighbours within the search radius (one
// lane each). The window ends at expeRT's upper cut (the 87 % rule,
// expeRT.cpp:662-676), the line is the FP32 least-squares fit over the
// window, and e = 10^(line at the top hit's bin) * cpsms
// (dslim_query.cpp:786-799). Where no bin is confirmed, or a level lies
// within FP32 rounding of a point, the spectrum is listed and the FP64
// expeRT fit (k_tailfit) runs on that list only.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "hc_device.cuh"
#include "hc_internal.h"

namespace hc {
namespace {

constexpr int kIn = 256, kH1 = 128, kH2 = 64, kOut = 4;
constexpr size_t kOffW1 = 0, kOffB1 = kOffW1 + kIn * kH1, kOffW2 = kOffB1 + kH1, kOffB2 = kOffW2 + kH1 * kH2,
                 kOffW3 = kOffB2 + kH2, kOffB3 = kOffW3 + kH2 * kOut, kParams = kOffB3 + kOut;
// target scaling: slope x 10, intercept / 4, first bin / 10, residual x 5
__host__ __device__ constexpr float tscale(int j)
{
    return j == 0 ? 10.0f : (j == 1 ? 0.25f : (j == 2 ? 0.1f : 5.0f));
}
// a 22 % or 87 % level closer than this to a curve point (log10 units) is a
// near tie the FP32 curve cannot decide the way expeRT's FP64 curve does
constexpr float kLevelMargin = 1e-4f;
constexpr int kMaxRadius = 15;  // first bins tested around the prediction: 2 * radius + 1 <= 32 lanes

}  // namespace
}  // namespace hc

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
    // gate of the learned tail: largest predicted RMS residual (log10 units),
    // and how far from the predicted first bin the confirmation looks
    float gate_resid = 0.1f;
    uint32_t radius = 4;
    // pipeline scratch (grown before any capture): features, outputs, fallback list
    float *d_X = nullptr, *d_net = nullptr;
    uint32_t *d_fb = nullptr;  // [0] = count, then the list
    size_t pipe_cap = 0;
};

namespace hc {
namespace {

// ---- features -------------------------------------------------------------
__global__ void k_features(const uint32_t *__restrict__ hist, const hc_result *__restrict__ res, uint32_t n,
                           float *__restrict__ X)
{
    const uint32_t s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= n) return;
    const uint32_t *h = hist + (size_t)s * HC_HIST_BINS;
    const hc_result r = res[s];
    const uint32_t cpi = r.cpsms > 0 ? r.cpsms : 1u;
    const float inv = 1.0f / (float)cpi;
    int hyp = hist_bin(r.hyperscore);
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
        // 1 - cumsum / cpsms from the exact integer difference
        const float sv = (float)(cpi - min(cpi, carry + v)) * inv;
        x[b] = log10f(fmaxf(sv, 1e-7f));
        carry += __shfl_sync(0xFFFFFFFFu, v, 31);
    }
    __syncwarp();
    // bins at/after the top hit's bin repeat the last value below it
    const float last = hyp > 0 ? x[hyp - 1] : 0.0f;
    __syncwarp();
    for (int b = hyp + lane; b < kIn; b += 32) x[b] = last;
}

// ---- dense layers for training (row-major: Y[n,N] = X[n,K] W[K,N] + b) ----
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

// MSE on scaled targets, NaN targets excluded: dOut = 2 (out - t) / (n * 4)
__global__ void k_mse(const float *__restrict__ out, const float *__restrict__ Y, int n, float *__restrict__ dOut,
                      float *__restrict__ loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < n * kOut)
    {
        const float y = Y[i];
        float d = 0.0f;
        if (!isnan(y)) d = out[i] - y * tscale(i % kOut);
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

// ---- inference: the three layers fused, weights resident in shared memory ----
// A CTA stages all parameters (about 162 KB) once and its warps then walk the
// spectra, two per warp at a time: lane j computes hidden units 4j..4j+3 of
// layer 1 (one 16-byte weight load per input serves both spectra) and 2j,
// 2j+1 of layer 2; the four outputs are warp sums. Activations stay in the
// warp's own shared-memory rows.
constexpr int kInferWarps = 8;
constexpr size_t kInferWeights = kParams;  // floats
constexpr size_t kInferSmem = 4 * (kInferWeights + (size_t)kInferWarps * 2 * (kIn + kH1 + kH2));

__global__ void __launch_bounds__(kInferWarps * 32) k_mlp_infer(const float *__restrict__ P,
                                                                const float *__restrict__ X, uint32_t n,
                                                                float *__restrict__ out)
{
    extern __shared__ __align__(16) float sm[];
    float *W = sm;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (size_t i = tid; i < kParams / 4; i += blockDim.x)
        reinterpret_cast<float4 *>(W)[i] = __ldg(reinterpret_cast<const float4 *>(P) + i);
    __syncthreads();
    const float *W1 = W + kOffW1, *b1 = W + kOffB1, *W2 = W + kOffW2, *b2 = W + kOffB2, *W3 = W + kOffW3,
                *b3 = W + kOffB3;
    float *xs = sm + kInferWeights + (size_t)warp * 2 * (kIn + kH1 + kH2);  // x[2][256] | h1[2][128] | h2[2][64]
    float *h1s = xs + 2 * kIn, *h2s = h1s + 2 * kH1;
    const uint32_t npair = (n + 1) / 2;
    for (uint32_t pr = blockIdx.x * kInferWarps + warp; pr < npair; pr += gridDim.x * kInferWarps)
    {
        const uint32_t s0 = 2 * pr, s1 = min(s0 + 1, n - 1);
        // inputs: 64 float4 per spectrum
        for (int i = lane; i < 2 * kIn / 4; i += 32)
        {
            const uint32_t sp = i < kIn / 4 ? s0 : s1;
            const int k = i % (kIn / 4);
            reinterpret_cast<float4 *>(xs)[i] = __ldg(reinterpret_cast<const float4 *>(X + (size_t)sp * kIn) + k);
        }
        __syncwarp();
        // layer 1: units 4*lane .. 4*lane + 3
        float4 a0 = reinterpret_cast<const float4 *>(b1)[lane], a1 = a0;
#pragma unroll 8
        for (int k = 0; k < kIn; k++)
        {
            const float4 w = reinterpret_cast<const float4 *>(W1 + (size_t)k * kH1)[lane];
            const float x0 = xs[k], x1 = xs[kIn + k];
            a0.x = fmaf(x0, w.x, a0.x); a0.y = fmaf(x0, w.y, a0.y); a0.z = fmaf(x0, w.z, a0.z); a0.w = fmaf(x0, w.w, a0.w);
            a1.x = fmaf(x1, w.x, a1.x); a1.y = fmaf(x1, w.y, a1.y); a1.z = fmaf(x1, w.z, a1.z); a1.w = fmaf(x1, w.w, a1.w);
        }
        reinterpret_cast<float4 *>(h1s)[lane] =
            make_float4(fmaxf(a0.x, 0.f), fmaxf(a0.y, 0.f), fmaxf(a0.z, 0.f), fmaxf(a0.w, 0.f));
        reinterpret_cast<float4 *>(h1s + kH1)[lane] =
            make_float4(fmaxf(a1.x, 0.f), fmaxf(a1.y, 0.f), fmaxf(a1.z, 0.f), fmaxf(a1.w, 0.f));
        __syncwarp();
        // layer 2: units 2*lane, 2*lane + 1
        float2 c0 = reinterpret_cast<const float2 *>(b2)[lane], c1 = c0;
#pragma unroll 8
        for (int k = 0; k < kH1; k++)
        {
            const float2 w = reinterpret_cast<const float2 *>(W2 + (size_t)k * kH2)[lane];
            const float x0 = h1s[k], x1 = h1s[kH1 + k];
            c0.x = fmaf(x0, w.x, c0.x); c0.y = fmaf(x0, w.y, c0.y);
            c1.x = fmaf(x1, w.x, c1.x); c1.y = fmaf(x1, w.y, c1.y);
        }
        reinterpret_cast<float2 *>(h2s)[lane] = make_float2(fmaxf(c0.x, 0.f), fmaxf(c0.y, 0.f));
        reinterpret_cast<float2 *>(h2s + kH2)[lane] = make_float2(fmaxf(c1.x, 0.f), fmaxf(c1.y, 0.f));
        __syncwarp();
        // layer 3: inputs lane and lane + 32, warp sums
        float o0[kOut], o1[kOut];
#pragma unroll
        for (int j = 0; j < kOut; j++)
        {
            const float wa = W3[lane * kOut + j], wb = W3[(lane + 32) * kOut + j];
            o0[j] = h2s[lane] * wa + h2s[lane + 32] * wb;
            o1[j] = h2s[kH2 + lane] * wa + h2s[kH2 + lane + 32] * wb;
        }
#pragma unroll
        for (int j = 0; j < kOut; j++)
        {
            for (int o = 16; o > 0; o >>= 1)
            {
                o0[j] += __shfl_xor_sync(0xFFFFFFFFu, o0[j], o);
                o1[j] += __shfl_xor_sync(0xFFFFFFFFu, o1[j], o);
            }
        }
        if (lane < kOut) out[(size_t)s0 * kOut + lane] = o0[lane] + b3[lane];
        if (lane < kOut && s1 != s0) out[(size_t)s1 * kOut + lane] = o1[lane] + b3[lane];
        __syncwarp();
    }
}

// ---- the learned tail ---------------------------------------------------------
constexpr int kLtWarps = 4;
enum TailMode
{
    kApply = 0,     // gated: learned spectra written, the others listed for expeRT
    kProbe = 1,     // every spectrum's learned value, no gate, nothing written to the results
    kBaseline = 2,  // as kProbe with no network: the search starts at the curve's first bin
    kExact = 3,     // expeRT's own window by a full search: the training targets
};

struct TailGate
{
    float max_resid;  // largest predicted RMS residual of a learned spectrum
    int radius;       // first bins tested on either side of the prediction
};

// One warp per spectrum. net: the network's outputs (n x 4, scaled). lg_out
// (optional): the learned log10 e-value (NaN where there is none; in kApply
// also where the spectrum went to expeRT). aux_out (optional, kProbe and
// kBaseline): per spectrum {predicted residual, residual of the fit, offset
// of the confirmed first bin from the prediction} (NaN where none). y_out
// (kExact): the training targets {slope, intercept, first bin, residual}
// (NaN where there is no fit).
__global__ void __launch_bounds__(kLtWarps * 32) k_learned_tail(const uint32_t *__restrict__ hist,
                                                                const float *__restrict__ net,
                                                                hc_result *__restrict__ res, uint32_t n,
                                                                TailGate gate, uint32_t min_cpsm,
                                                                double expect_max, int mode,
                                                                float *__restrict__ lg_out,
                                                                float *__restrict__ aux_out,
                                                                float *__restrict__ y_out,
                                                                uint32_t *__restrict__ fb)
{
    __shared__ float ys[kLtWarps][HC_HIST_BINS + 2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float *y = ys[warp];
    const float nanf_ = __int_as_float(0x7FC00000);
    for (uint32_t s = blockIdx.x * kLtWarps + warp; s < n; s += gridDim.x * kLtWarps)
    {
        hc_result r = res[s];
        const float presid = (net && mode != kBaseline) ? net[(size_t)s * kOut + 3] / tscale(3) : nanf_;
        const bool early_fb = mode == kApply && !(presid <= gate.max_resid);
        if (r.cpsms < min_cpsm || r.cpsms == 0 || early_fb)
        {
            if (lane == 0)
            {
                if (mode == kApply && !early_fb)
                {
                    // no e-value (the early return of the tail fit, dslim_query.cpp:773)
                    r.mu = r.beta = r.minhyp = r.nexthyp = r.maxhyp = 0;
                    r.evalue = 0.0;
                    r.reported = 0;
                    res[s] = r;
                }
                if (early_fb) fb[1 + atomicAdd(fb, 1u)] = s;
                if (lg_out) lg_out[s] = nanf_;
                if (aux_out) aux_out[3 * s] = presid, aux_out[3 * s + 1] = aux_out[3 * s + 2] = nanf_;
                if (y_out) y_out[4 * s] = y_out[4 * s + 1] = y_out[4 * s + 2] = y_out[4 * s + 3] = nanf_;
            }
            continue;
        }
        const uint32_t *yy = hist + (size_t)s * HC_HIST_BINS;
        const int hyp = hist_bin(r.hyperscore);
        const uint32_t cps = r.cpsms;
        int stt1, end1;
        const int nb = tail_bins(yy, hyp, HC_HIST_BINS, lane, stt1, end1);
        bool have = false;
        int mark = 0, offset = 0;
        float slope = 0.0f, icpt = 0.0f, resid = nanf_;
        if (nb >= 4)
        {
            // survival curve log10((cpsms - cumsum) / cpsms) over [stt1, end1]:
            // the difference is an exact integer, positive below the top hit,
            // and the curve does not increase
            uint32_t carry = 0;
            const float inv = 1.0f / (float)cps;
            for (int i0 = 0; i0 < nb; i0 += 32)
            {
                const int i = i0 + lane;
                uint32_t v = (i < nb) ? yy[stt1 + i] : 0u;
                for (int o = 1; o < 32; o <<= 1)
                {
                    const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, v, o);
                    if (lane >= o) v += t;
                }
                if (i < nb)
                {
                    const uint32_t left = cps - min(cps, carry + v);
                    y[i] = log10f(fmaxf((float)left * inv, 1e-9f));
                }
                carry += __shfl_sync(0xFFFFFFFFu, v, 31);
            }
            __syncwarp();
            const float y0 = y[0], hgt = y[nb - 1] - y0;
            // upper end (expeRT.cpp:662-676): the last point at or above the 87 % level
            const float t2 = y0 + 0.87f * hgt;
            int m2 = nb - 1;
            for (int q0 = nb - 1; q0 >= 0; q0 -= 32)
            {
                const int q = q0 - lane;
                const uint32_t b = __ballot_sync(0xFFFFFFFFu, q >= 0 && y[q] >= t2);
                if (b)
                {
                    m2 = q0 - (__ffs(b) - 1);
                    break;
                }
            }
            bool clear = fabsf(y[m2] - t2) > kLevelMargin && (m2 + 1 >= nb || fabsf(y[m2 + 1] - t2) > kLevelMargin);
            // first bin: the point before the first one at or below the 22 % level
            const float t1 = y0 + 0.22f * hgt;
            int lm = -1;  // the first point at or below t1
            if (mode == kExact)
            {
                for (int q0 = 0; q0 < nb; q0 += 32)
                {
                    const int q = q0 + lane;
                    const uint32_t b = __ballot_sync(0xFFFFFFFFu, q < nb && y[q] <= t1);
                    if (b)
                    {
                        lm = q0 + __ffs(b) - 1;
                        break;
                    }
                }
            }
            else
            {
                // lane j tests lm = center + j - radius: y[lm] <= t1 < y[lm - 1]
                const int center = mode == kBaseline ? 1 : (int)lrintf(net[(size_t)s * kOut + 2] / tscale(2)) - stt1 + 1;
                const int q = center + lane - gate.radius;
                const bool hit = lane <= 2 * gate.radius && q >= 0 && q < nb && y[q] <= t1 && (q == 0 || y[q - 1] > t1);
                const uint32_t b = __ballot_sync(0xFFFFFFFFu, hit);
                if (b)
                {
                    const int j = __ffs(b) - 1;
                    lm = center + j - gate.radius;
                    offset = j - gate.radius;
                }
            }
            if (lm >= 0)
                clear = clear && fabsf(y[lm] - t1) > kLevelMargin && (lm == 0 || fabsf(y[lm - 1] - t1) > kLevelMargin);
            mark = min(lm - 1, m2 - 1);
            // a window starting before the curve reads element -1 in the
            // reference (flagged): left to expeRT, as are near ties
            if (lm >= 0 && mark >= 0 && clear)
            {
                const int first = mark, m = m2 - first + 1;
                const float xbar = 0.5f * (float)(first + m2);  // window-relative abscissae
                float sy = 0.0f;
                for (int i = lane; i < m; i += 32) sy += y[first + i];
                for (int o = 16; o > 0; o >>= 1) sy += __shfl_xor_sync(0xFFFFFFFFu, sy, o);
                const float ybar = sy / (float)m;
                float top = 0.0f, bot = 0.0f;
                for (int i = lane; i < m; i += 32)
                {
                    const float dx = (float)(first + i) - xbar;
                    top = fmaf(dx, y[first + i] - ybar, top);
                    bot = fmaf(dx, dx, bot);
                }
                for (int o = 16; o > 0; o >>= 1)
                {
                    top += __shfl_xor_sync(0xFFFFFFFFu, top, o);
                    bot += __shfl_xor_sync(0xFFFFFFFFu, bot, o);
                }
                const float sl = top / bot;
                float se = 0.0f;
                for (int i = lane; i < m; i += 32)
                {
                    const float d = fmaf(sl, (float)(first + i) - xbar, ybar) - y[first + i];
                    se = fmaf(d, d, se);
                }
                for (int o = 16; o > 0; o >>= 1) se += __shfl_xor_sync(0xFFFFFFFFu, se, o);
                slope = sl;
                // intercept in histogram bins: the line is ybar + sl (bin - stt1 - xbar)
                icpt = ybar - sl * ((float)stt1 + xbar);
                resid = sqrtf(se / (float)m);
                have = isfinite(slope) && isfinite(icpt);
            }
            __syncwarp();
        }
        if (lane == 0)
        {
            // e(x) from the line as the reference forms it from expeRT's (mu, beta)
            // (x 1e6, truncated to int; dslim_query.cpp:786-799)
            const int32_t mu = x86_d2i((double)slope * 1e6), beta = x86_d2i((double)icpt * 1e6);
            const double lgs = (double)mu / 1e6 * (double)hyp + (double)beta / 1e6;
            const double lg = lgs + log10((double)cps);
            if (lg_out) lg_out[s] = have ? (float)lg : nanf_;
            if (aux_out)
            {
                aux_out[3 * s] = presid;
                aux_out[3 * s + 1] = have ? resid : nanf_;
                aux_out[3 * s + 2] = have ? (float)offset : nanf_;
            }
            if (y_out)
            {
                y_out[4 * s] = have ? slope : nanf_;
                y_out[4 * s + 1] = have ? icpt : nanf_;
                y_out[4 * s + 2] = have ? (float)(stt1 + mark) : nanf_;
                y_out[4 * s + 3] = have ? resid : nanf_;
            }
            if (mode == kApply)
            {
                if (have)
                {
                    r.mu = mu;
                    r.beta = beta;
                    r.minhyp = stt1;
                    r.nexthyp = end1;
                    r.maxhyp = hyp;
                    r.evalue = pow(10.0, lgs) * (double)cps;
                    r.reported = r.evalue < expect_max ? 1u : 0u;
                    r.flags |= HC_FLAG_LEARNED;
                    res[s] = r;
                }
                else
                    fb[1 + atomicAdd(fb, 1u)] = s;  // the expeRT fit runs on it
            }
        }
        __syncwarp();
    }
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

// the fused inference kernel (no activations kept)
static int mlp_infer(hc_mlp *m, const float *X, uint32_t n, float *out, cudaStream_t st)
{
    if (n == 0) return HC_SUCCESS;
    static_assert(kParams % 4 == 0, "parameters are staged as float4");
    HC_CUDA(m->ctx, cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem));
    const uint32_t pairs = (n + 1) / 2;
    const uint32_t blocks = std::min<uint32_t>((pairs + kInferWarps - 1) / kInferWarps, (uint32_t)m->ctx->sm_count);
    k_mlp_infer<<<blocks, kInferWarps * 32, kInferSmem, st>>>(m->d_params, X, n, out);
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

static int grow_pipe(hc_mlp *m, uint32_t n)
{
    if (m->pipe_cap >= n) return HC_SUCCESS;
    cudaFree(m->d_X);
    cudaFree(m->d_net);
    cudaFree(m->d_fb);
    m->d_X = m->d_net = nullptr;
    m->d_fb = nullptr;
    m->pipe_cap = 0;
    HC_CUDA(m->ctx, cudaMalloc((void **)&m->d_X, sizeof(float) * kIn * (size_t)n));
    HC_CUDA(m->ctx, cudaMalloc((void **)&m->d_net, sizeof(float) * kOut * (size_t)n));
    HC_CUDA(m->ctx, cudaMalloc((void **)&m->d_fb, sizeof(uint32_t) * ((size_t)n + 1)));
    m->pipe_cap = n;
    return HC_SUCCESS;
}

static int tail_kernel(hc_ctx *ctx, const TailGate &g, const uint32_t *d_hist, const float *net, hc_result *d_res,
                       uint32_t n, int mode, float *lg, float *aux, float *y, uint32_t *fb, cudaStream_t st)
{
    if (n == 0) return HC_SUCCESS;
    const uint32_t blocks = std::min<uint32_t>((n + kLtWarps - 1) / kLtWarps, (uint32_t)ctx->sm_count * 16);
    k_learned_tail<<<blocks, kLtWarps * 32, 0, st>>>(d_hist, net, d_res, n, g, ctx->p.min_cpsm, ctx->p.expect_max,
                                                     mode, lg, aux, y, fb);
    HC_CUDA(ctx, cudaGetLastError());
    return HC_SUCCESS;
}

static TailGate gate_of(const hc_mlp *m) { return TailGate{m->gate_resid, (int)m->radius}; }

void learned_gate(const hc_mlp *m, float *max_resid, uint32_t *radius)
{
    *max_resid = m->gate_resid;
    *radius = m->radius;
}

// Allocates what the learned pipeline of n spectra needs (before any capture).
int learned_prepare(hc_mlp *m, uint32_t n)
{
    int rc = grow_pipe(m, n);
    if (rc) return rc;
    QueryScratch &q = m->ctx->qs;
    if (q.fit_cap < n)
    {
        cudaFree(q.d_fitstart);
        q.d_fitstart = nullptr;
        q.fit_cap = 0;
        HC_CUDA(m->ctx, cudaMalloc((void **)&q.d_fitstart, sizeof(int32_t) * (size_t)n));
        q.fit_cap = n;
    }
    return HC_SUCCESS;
}

// After a search without tail fit: features, network, learned e-values where
// the gates pass, and expeRT's fit on the listed rest. Enqueue only (no
// allocation after learned_prepare, no host wait). lg (optional) receives the
// learned log10 e-values.
int learned_pipeline(hc_mlp *m, const uint32_t *d_hist, hc_result *d_res, uint32_t n, float *lg, cudaStream_t st,
                     int *launches)
{
    if (n == 0) return HC_SUCCESS;
    if (m->pipe_cap < n || m->ctx->qs.fit_cap < n)
        return set_error(m->ctx, HC_ERR_INVLD_SIZE, "learned pipeline scratch not prepared");
    HC_CUDA(m->ctx, cudaMemsetAsync(m->d_fb, 0, 4, st));
    k_features<<<(n + 3) / 4, 128, 0, st>>>(d_hist, d_res, n, m->d_X);
    HC_CUDA(m->ctx, cudaGetLastError());
    int rc = mlp_infer(m, m->d_X, n, m->d_net, st);
    if (rc) return rc;
    if ((rc = tail_kernel(m->ctx, gate_of(m), d_hist, m->d_net, d_res, n, kApply, lg, nullptr, nullptr, m->d_fb,
                          st)))
        return rc;
    if ((rc = tailfit_list(m->ctx, d_res, d_hist, m->d_fb + 1, m->d_fb, n, st))) return rc;
    if (m->ctx->profiling) HC_CUDA(m->ctx, record_stage(m->ctx, 5, st));
    if (launches) *launches += 4;
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
        hc_mlp_destroy(m);
        return HC_ERR_BAD_MEM_ALLOC;
    }
    if (cudaMemcpy(m->d_params, h.data(), 4 * kParams, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(m->d_m, 0, 4 * kParams) != cudaSuccess || cudaMemset(m->d_v, 0, 4 * kParams) != cudaSuccess)
    {
        hc_mlp_destroy(m);
        return HC_ERR_CUDA;
    }
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
    cudaFree(m->d_X);
    cudaFree(m->d_net);
    cudaFree(m->d_fb);
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

int hc_mlp_set_gate(hc_mlp *m, float max_resid, uint32_t radius)
{
    if (!m) return HC_ERR_INVLD_PTR;
    if (radius > (uint32_t)kMaxRadius || !(max_resid >= 0.0f)) return set_error(m->ctx, HC_ERR_INVLD_PARAM, "bad gate");
    m->gate_resid = max_resid;
    m->radius = radius;
    return HC_SUCCESS;
}

int hc_mlp_get_gate(const hc_mlp *m, float *max_resid, uint32_t *radius)
{
    if (!m) return HC_ERR_INVLD_PTR;
    if (max_resid) *max_resid = m->gate_resid;
    if (radius) *radius = m->radius;
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

int hc_mlp_targets(hc_ctx *ctx, const uint32_t *d_hist, const hc_result *d_res, uint32_t n, float *d_Y, void *stream)
{
    if (!ctx || (n && (!d_hist || !d_res || !d_Y))) return HC_ERR_INVLD_PTR;
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    return tail_kernel(ctx, TailGate{0.0f, 0}, d_hist, nullptr, const_cast<hc_result *>(d_res), n, kExact, nullptr,
                       nullptr, d_Y, nullptr, st);
}

int hc_mlp_forward(hc_mlp *m, const float *d_X, uint32_t n, float *d_out, void *stream)
{
    if (!m || (n && (!d_X || !d_out))) return HC_ERR_INVLD_PTR;
    cudaStream_t st = stream ? (cudaStream_t)stream : m->ctx->stream;
    return mlp_infer(m, d_X, n, d_out, st);
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

int hc_mlp_tail_probe(hc_mlp *m, const float *d_X, const uint32_t *d_hist, const hc_result *d_res, uint32_t n,
                      int baseline, float *d_learned_log10e, float *d_aux, void *stream)
{
    if (!m || (n && (!d_hist || !d_res || !d_learned_log10e || !d_aux || (!baseline && !d_X)))) return HC_ERR_INVLD_PTR;
    cudaStream_t st = stream ? (cudaStream_t)stream : m->ctx->stream;
    if (n == 0) return HC_SUCCESS;
    int rc = grow_pipe(m, n);
    if (rc) return rc;
    const float *net = nullptr;
    if (!baseline)
    {
        if ((rc = mlp_infer(m, d_X, n, m->d_net, st))) return rc;
        net = m->d_net;
    }
    return tail_kernel(m->ctx, gate_of(m), d_hist, net, const_cast<hc_result *>(d_res), n,
                       baseline ? kBaseline : kProbe, d_learned_log10e, d_aux, nullptr, nullptr, st);
}

}  // extern "C"
