// The learned closure's network outside the step: host packing of lbm_closure_t into the per-lane
// tensor-core fragments the collision reads, and the float32 training kernels (forward, backward,
// Adam) over feature rows.  No counterpart in the reference (its LES is Smagorinsky only,
// src/lbm/kernels/ops/turbulence.mojo:12-38).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>

#include "lbm_closure.cuh"

namespace lbm {

__attribute__((visibility("hidden"))) void set_last_error(const char* msg);

namespace {

constexpr int kIn = 8, kHid = 32;
constexpr int kW1 = 0, kB1 = kW1 + kIn * kHid, kW2 = kB1 + kHid, kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid,
              kB3 = kW3 + kHid, kParams = kB3 + 1;
static_assert(kParams == 1377, "theta packing: w1, b1, w2, b2, w3, b3");

// float -> bfloat16 bits, round to nearest even (NaN kept quiet).
uint16_t bf16_bits(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7FFFFFFFu) > 0x7F800000u) return 0x7FC0u;
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

uint32_t pair(float lo, float hi) { return (uint32_t)bf16_bits(lo) | ((uint32_t)bf16_bits(hi) << 16); }

// ---- training kernels -------------------------------------------------------------------------

constexpr int kFwdThreads = 256;
constexpr int kBwdThreads = 128;   // one sample per thread per chunk
constexpr int kPad = kHid + 1;                // padded row of a hidden-layer array in shared memory
constexpr int kBwdRow = kIn + 4 * kPad + 1;   // x, h1, dh1, gy*h2, dh2, gy per sample

__device__ __forceinline__ void load_theta(const float* __restrict__ theta, float* w) {
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = theta[i];
    __syncthreads();
}

// acc[j] += a * w[j] for 32 consecutive weights (shared memory, 16-byte aligned: broadcast reads).
__device__ __forceinline__ void axpy32(float (&acc)[kHid], float a, const float* w) {
#pragma unroll
    for (int j = 0; j < kHid; j += 4) {
        const float4 v = *reinterpret_cast<const float4*>(w + j);
        acc[j] = __fmaf_rn(a, v.x, acc[j]);
        acc[j + 1] = __fmaf_rn(a, v.y, acc[j + 1]);
        acc[j + 2] = __fmaf_rn(a, v.z, acc[j + 2]);
        acc[j + 3] = __fmaf_rn(a, v.w, acc[j + 3]);
    }
}

// One sample through the network: h1, h2 (after ReLU) and the pre-activation output y.
__device__ __forceinline__ float mlp_forward_one(const float* w, const float (&x)[kIn], float (&h1)[kHid],
                                                 float (&h2)[kHid]) {
#pragma unroll
    for (int j = 0; j < kHid; ++j) h1[j] = w[kB1 + j];
#pragma unroll
    for (int k = 0; k < kIn; ++k) axpy32(h1, x[k], w + kW1 + k * kHid);
#pragma unroll
    for (int j = 0; j < kHid; ++j) {
        h1[j] = fmaxf(h1[j], 0.f);
        h2[j] = w[kB2 + j];
    }
#pragma unroll
    for (int k = 0; k < kHid; ++k) axpy32(h2, h1[k], w + kW2 + k * kHid);
    float y = w[kB3];
#pragma unroll
    for (int k = 0; k < kHid; ++k) {
        h2[k] = fmaxf(h2[k], 0.f);
        y = __fmaf_rn(h2[k], w[kW3 + k], y);
    }
    return y;
}

__device__ __forceinline__ float softplus(float y) { return y > 20.f ? y : log1pf(expf(y)); }

__global__ void __launch_bounds__(kFwdThreads) mlp_forward_kernel(const float* __restrict__ theta,
                                                                  const float* __restrict__ x, int64_t n,
                                                                  float nu_scale, float* __restrict__ nu) {
    __shared__ __align__(16) float w[kParams];
    load_theta(theta, w);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        // keeps the weight reads inside the loop (hoisted, 1377 weights would not fit in registers)
        asm volatile("" ::: "memory");
        float xi[kIn], h1[kHid], h2[kHid];
#pragma unroll
        for (int k = 0; k < kIn; ++k) xi[k] = x[i * kIn + k];
        nu[i] = softplus(mlp_forward_one(w, xi, h1, h2)) * nu_scale;
    }
}

// Per-block partial gradients over a contiguous range of samples, in chunks of kBwdThreads.  Each
// thread recomputes its sample's activations, leaves x, h1, dh1, gy*h2, dh2 and gy in shared
// memory, and then owns fixed parameters whose sums over the chunk it accumulates in registers
// (a warp's lanes read consecutive hidden units, the same sample row: no bank conflicts).
__global__ void __launch_bounds__(kBwdThreads) mlp_backward_kernel(const float* __restrict__ theta,
                                                                   const float* __restrict__ x,
                                                                   const float* __restrict__ g, int64_t n,
                                                                   float nu_scale, int64_t per_block,
                                                                   float* __restrict__ partial) {
    __shared__ __align__(16) float w[kParams];
    extern __shared__ float rows[];  // kBwdThreads * kBwdRow
    load_theta(theta, w);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float* X = rows;
    float* H1 = X + kBwdThreads * kIn;
    float* DH1 = H1 + kBwdThreads * kPad;
    float* P3 = DH1 + kBwdThreads * kPad;
    float* DH2 = P3 + kBwdThreads * kPad;
    float* GY = DH2 + kBwdThreads * kPad;

    float acc_w2[8], acc_w1[2], acc_x = 0.f;
#pragma unroll
    for (int r = 0; r < 8; ++r) acc_w2[r] = 0.f;
    acc_w1[0] = acc_w1[1] = 0.f;

    const int64_t s0 = (int64_t)blockIdx.x * per_block;
    const int64_t s1 = s0 + per_block < n ? s0 + per_block : n;
    for (int64_t c = s0; c < s1; c += kBwdThreads) {
        asm volatile("" ::: "memory");  // keeps the weight reads inside the loop
        const int64_t i = c + tid;
        float xi[kIn], h1[kHid], h2[kHid];
        float gy = 0.f;
        if (i < s1) {
#pragma unroll
            for (int k = 0; k < kIn; ++k) xi[k] = x[i * kIn + k];
            const float y = mlp_forward_one(w, xi, h1, h2);
            gy = g[i] * nu_scale / (1.f + expf(-y));  // d softplus / dy = sigmoid(y)
        } else {
#pragma unroll
            for (int k = 0; k < kIn; ++k) xi[k] = 0.f;
#pragma unroll
            for (int k = 0; k < kHid; ++k) h1[k] = h2[k] = 0.f;
        }
        float dh2[kHid];
#pragma unroll
        for (int k = 0; k < kIn; ++k) X[tid * kIn + k] = xi[k];
#pragma unroll
        for (int j = 0; j < kHid; ++j) {
            dh2[j] = h2[j] > 0.f ? gy * w[kW3 + j] : 0.f;
            H1[tid * kPad + j] = h1[j];
            P3[tid * kPad + j] = gy * h2[j];
            DH2[tid * kPad + j] = dh2[j];
        }
#pragma unroll 1
        for (int j = 0; j < kHid; ++j) {  // dh1 = (W2 dh2) masked by ReLU
            float a = 0.f;
#pragma unroll
            for (int k = 0; k < kHid; k += 4) {
                const float4 v = *reinterpret_cast<const float4*>(w + kW2 + j * kHid + k);
                a = __fmaf_rn(v.x, dh2[k], a);
                a = __fmaf_rn(v.y, dh2[k + 1], a);
                a = __fmaf_rn(v.z, dh2[k + 2], a);
                a = __fmaf_rn(v.w, dh2[k + 3], a);
            }
            DH1[tid * kPad + j] = H1[tid * kPad + j] > 0.f ? a : 0.f;
        }
        GY[tid] = gy;
        __syncthreads();
        const int rows_here = (int)((s1 - c) < kBwdThreads ? (s1 - c) : kBwdThreads);
        for (int s = 0; s < rows_here; ++s) {
            const float d2 = DH2[s * kPad + lane];
#pragma unroll
            for (int r = 0; r < 8; ++r) acc_w2[r] = __fmaf_rn(H1[s * kPad + warp + 4 * r], d2, acc_w2[r]);
            const float d1 = DH1[s * kPad + lane];
            acc_w1[0] = __fmaf_rn(X[s * kIn + warp], d1, acc_w1[0]);
            acc_w1[1] = __fmaf_rn(X[s * kIn + warp + 4], d1, acc_w1[1]);
            // warp 0: b1, warp 1: b2, warp 2: w3, warp 3: b3 (lane 0)
            acc_x += warp == 0 ? d1 : warp == 1 ? d2 : warp == 2 ? P3[s * kPad + lane] : GY[s];
        }
        __syncthreads();
    }
    float* out = partial + (size_t)blockIdx.x * kParams;
#pragma unroll
    for (int r = 0; r < 8; ++r) out[kW2 + (warp + 4 * r) * kHid + lane] = acc_w2[r];
    out[kW1 + warp * kHid + lane] = acc_w1[0];
    out[kW1 + (warp + 4) * kHid + lane] = acc_w1[1];
    if (warp == 0) out[kB1 + lane] = acc_x;
    else if (warp == 1) out[kB2 + lane] = acc_x;
    else if (warp == 2) out[kW3 + lane] = acc_x;
    else if (lane == 0) out[kB3] = acc_x;
}

// grad[p] = sum over blocks of partial[b][p], in block order (deterministic).
__global__ void mlp_sum_partials_kernel(const float* __restrict__ partial, int nblocks, float* __restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kParams) return;
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * kParams + p];
    grad[p] = s;
}

__global__ void mlp_adam_kernel(float* __restrict__ theta, const float* __restrict__ grad, float* __restrict__ m,
                                float* __restrict__ v, int n, float lr_t, float beta1, float beta2, float eps_t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = grad[i];
    const float mi = beta1 * m[i] + (1.f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    theta[i] -= lr_t * mi / (sqrtf(vi) + eps_t);
}

lbm_status fail(lbm_status s, const char* msg) {
    set_last_error(msg);
    return s;
}

lbm_status cuda_fail(const char* where, cudaError_t e) {
    static thread_local char buf[256];
    std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
    set_last_error(buf);
    return LBM_ECUDA;
}

int sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return 1;
    return sms;
}

}  // namespace

// Fills the per-lane fragments of m16n8k16 B operands (k rows 2t, 2t+1 in register 0 and
// 2t+8, 2t+9 in register 1 of column g, lane = 4g + t) and the accumulator bias pairs.
__attribute__((visibility("hidden"))) void pack_closure(const lbm_closure_t& c, ClosureDev& d, ClosureUniform& u) {
    std::memset(&d, 0, sizeof(d));
    std::memset(&u, 0, sizeof(u));
    for (int lane = 0; lane < 32; ++lane) {
        const int g = lane >> 2, t = lane & 3;
        for (int nt = 0; nt < 4; ++nt) {
            const int col = 8 * nt + g;
            d.w1f[nt][lane].x = pair(c.w1[(2 * t) * kHid + col], c.w1[(2 * t + 1) * kHid + col]);
            d.w1f[nt][lane].y = 0u;  // features 8..15 are the zero padding of K
            for (int kc = 0; kc < 2; ++kc) {
                const int k = 16 * kc + 2 * t;
                const uint32_t r0 = pair(c.w2[k * kHid + col], c.w2[(k + 1) * kHid + col]);
                const uint32_t r1 = pair(c.w2[(k + 8) * kHid + col], c.w2[(k + 9) * kHid + col]);
                if (kc == 0) { d.w2f[nt][lane].x = r0; d.w2f[nt][lane].y = r1; }
                else { d.w2f[nt][lane].z = r0; d.w2f[nt][lane].w = r1; }
            }
            const float b1x = c.b1[8 * nt + 2 * t], b1y = c.b1[8 * nt + 2 * t + 1];
            const float b2x = c.b2[8 * nt + 2 * t], b2y = c.b2[8 * nt + 2 * t + 1];
            d.b1q[nt][lane] = make_float4(b1x, b1y, b1x, b1y);
            d.b2q[nt][lane] = make_float4(b2x, b2y, b2x, b2y);
        }
        for (int kc = 0; kc < 2; ++kc) {
            const int k = 16 * kc + 2 * t;
            if (g == 0) {  // only output column 0 is used
                const uint32_t r0 = pair(c.w3[k], c.w3[k + 1]), r1 = pair(c.w3[k + 8], c.w3[k + 9]);
                if (kc == 0) { d.w3f[lane].x = r0; d.w3f[lane].y = r1; }
                else { d.w3f[lane].z = r0; d.w3f[lane].w = r1; }
            }
        }
    }
    for (int k = 0; k < 8; ++k) {
        u.scale[k] = c.feat_scale[k];
        u.shift[k] = -(c.feat_mean[k] * c.feat_scale[k]);  // x_n = fma(x, scale, shift)
        u.lo[k] = c.feat_lo[k];
        u.hi[k] = c.feat_hi[k];
    }
    d.b3q = make_float4(c.b3, c.b3, c.b3, c.b3);
    u.nu_scale = c.nu_scale;
}

}  // namespace lbm

using namespace lbm;

extern "C" {

lbm_status lbm_mlp_forward(const float* theta, const float* x, int64_t n, float nu_scale, float* nu, void* stream) {
    if (n < 0) return fail(LBM_EINVAL, "n must be non-negative");
    if (n == 0) return LBM_OK;
    if (!theta || !x || !nu) return fail(LBM_EINVAL, "null buffer");
    const int64_t want = (n + kFwdThreads - 1) / kFwdThreads;
    const int blocks = (int)(want < 8 * sm_count() ? want : 8 * sm_count());
    mlp_forward_kernel<<<blocks, kFwdThreads, 0, (cudaStream_t)stream>>>(theta, x, n, nu_scale, nu);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : cuda_fail("mlp_forward_kernel", e);
}

lbm_status lbm_mlp_backward(const float* theta, const float* x, const float* g, int64_t n, float nu_scale,
                            float* grad_theta, void* stream) {
    if (n < 0) return fail(LBM_EINVAL, "n must be non-negative");
    if (!theta || !grad_theta || (n > 0 && (!x || !g))) return fail(LBM_EINVAL, "null buffer");
    cudaStream_t s = (cudaStream_t)stream;
    if (n == 0) {
        const cudaError_t e = cudaMemsetAsync(grad_theta, 0, sizeof(float) * kParams, s);
        return e == cudaSuccess ? LBM_OK : cuda_fail("cudaMemsetAsync", e);
    }
    const int64_t chunks = (n + kBwdThreads - 1) / kBwdThreads;
    const int64_t max_blocks = 4 * (int64_t)sm_count();
    const int nblocks = (int)(chunks < max_blocks ? chunks : max_blocks);
    const int64_t per_block = ((chunks + nblocks - 1) / nblocks) * kBwdThreads;
    const int used = (int)((n + per_block - 1) / per_block);
    const size_t smem = sizeof(float) * kBwdThreads * kBwdRow;
    cudaError_t e = cudaFuncSetAttribute(mlp_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail("cudaFuncSetAttribute", e);
    float* partial = nullptr;
    e = cudaMallocAsync(&partial, sizeof(float) * kParams * used, s);
    if (e != cudaSuccess) return cuda_fail("cudaMallocAsync", e);
    mlp_backward_kernel<<<used, kBwdThreads, smem, s>>>(theta, x, g, n, nu_scale, per_block, partial);
    e = cudaGetLastError();
    if (e == cudaSuccess) {
        mlp_sum_partials_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(partial, used, grad_theta);
        e = cudaGetLastError();
    }
    const cudaError_t ef = cudaFreeAsync(partial, s);
    if (e != cudaSuccess) return cuda_fail("mlp_backward_kernel", e);
    return ef == cudaSuccess ? LBM_OK : cuda_fail("cudaFreeAsync", ef);
}

lbm_status lbm_mlp_adam(float* theta, const float* grad, float* m, float* v, int32_t n_params, float lr, float beta1,
                        float beta2, float eps, int32_t t, void* stream) {
    if (n_params < 0 || t < 1) return fail(LBM_EINVAL, "n_params must be non-negative and t >= 1");
    if (n_params == 0) return LBM_OK;
    if (!theta || !grad || !m || !v) return fail(LBM_EINVAL, "null buffer");
    // Kingma & Ba (ICLR 2015), Algorithm 1 with the bias corrections folded into the step size
    // and epsilon: lr_t = lr sqrt(1 - beta2^t) / (1 - beta1^t), eps_t = eps sqrt(1 - beta2^t).
    const double c1 = 1.0 - std::pow((double)beta1, t), c2 = std::sqrt(1.0 - std::pow((double)beta2, t));
    const float lr_t = (float)(lr * c2 / c1), eps_t = (float)(eps * c2);
    mlp_adam_kernel<<<(n_params + 255) / 256, 256, 0, (cudaStream_t)stream>>>(theta, grad, m, v, n_params, lr_t, beta1,
                                                                            beta2, eps_t);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? LBM_OK : cuda_fail("mlp_adam_kernel", e);
}

}  // extern "C"
