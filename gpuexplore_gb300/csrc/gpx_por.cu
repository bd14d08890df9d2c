// gpx_por.cu -- training of the learned cluster proposal (a 40-64-1 MLP) on the GPU.
//
// Kernels (one training step over a minibatch of B rows):
//   quantize_kernel   fp32 master weights -> fake-quantised int8-valued weights
//                     (per-row scale max|w|/127 for layer 1, one scale for layer 2)
//   forward_kernel    one thread per row: pre = W1q (x/16) + b1 (fp32 FMA, j in
//                     order), h = bf16(relu(pre)), out = W2q h + b2, squared error
//   hidden_grad_kernel dpre = dout * W2q * [pre > 0] (straight-through the int8 and
//                     bf16 roundings)
//   grad_w1_kernel    one block per hidden unit: dW1[k] = sum_rows dpre[k] x/16, db1
//   grad_w2_kernel    dW2 = sum_rows h dout, db2 = sum_rows dout
//   adam_kernel       Adam with decoupled weight decay on the master weights
// gpx_por_grad runs one quantize/forward/backward without the update so the
// gradients can be checked against a CPU reference.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "gpx.h"

namespace gpx {
namespace {

constexpr int F = GPX_POR_FEATURES;
constexpr int H = GPX_POR_HIDDEN;
constexpr int NW = H * F + H + H + 1; // w1, b1, w2, b2
constexpr float kInScale = 1.0f / 16.0f;

__host__ __device__ inline float bf16_rne(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    memcpy(&f, &u, 4);
    return f;
}

// w = [w1 (H*F) | b1 (H) | w2 (H) | b2]; q receives the fake-quantised copy and scales
__global__ void quantize_kernel(const float *w, float *q, float *scales) {
    int k = threadIdx.x;
    if (k < H) {
        float m = 0;
        for (int j = 0; j < F; j++) m = fmaxf(m, fabsf(w[k * F + j]));
        float s = m > 0 ? m / 127.0f : 1e-8f;
        for (int j = 0; j < F; j++) q[k * F + j] = rintf(fminf(127.0f, fmaxf(-127.0f, w[k * F + j] / s))) * s;
        scales[k] = s;
        q[H * F + k] = w[H * F + k];
    }
    __syncthreads();
    if (k == 0) {
        float m = 0;
        for (int j = 0; j < H; j++) m = fmaxf(m, fabsf(w[H * F + H + j]));
        float s = m > 0 ? m / 127.0f : 1e-8f;
        for (int j = 0; j < H; j++)
            q[H * F + H + j] = rintf(fminf(127.0f, fmaxf(-127.0f, w[H * F + H + j] / s))) * s;
        scales[H] = s;
        q[NW - 1] = w[NW - 1];
    }
}

__global__ void forward_kernel(const uint8_t *x, const float *y, uint32_t rows, const float *q, float *pre,
                               float *hid, float *dout, float *loss) {
    __shared__ float sq[NW];
    for (int i = threadIdx.x; i < NW; i += blockDim.x) sq[i] = q[i];
    __syncthreads();
    uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    float err2 = 0;
    if (r < rows) {
        float xs[F];
        for (int j = 0; j < F; j++) xs[j] = (float)x[(size_t)r * F + j] * kInScale;
        float out = 0;
        for (int k = 0; k < H; k++) {
            float a = sq[H * F + k];
            for (int j = 0; j < F; j++) a = fmaf(sq[k * F + j], xs[j], a);
            float h = bf16_rne(a > 0 ? a : 0.0f);
            pre[(size_t)r * H + k] = a;
            hid[(size_t)r * H + k] = h;
            out = fmaf(sq[H * F + H + k], h, out);
        }
        out += sq[NW - 1];
        float e = out - y[r];
        dout[r] = 2.0f * e / (float)rows;
        err2 = e * e;
    }
    for (int o = 16; o; o >>= 1) err2 += __shfl_xor_sync(0xFFFFFFFFu, err2, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, err2 / (float)rows);
}

__global__ void hidden_grad_kernel(uint32_t rows, const float *q, const float *pre, const float *dout, float *dpre) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= (size_t)rows * H) return;
    int k = (int)(i % H);
    float g = dout[i / H] * q[H * F + H + k];
    dpre[i] = pre[i] > 0 ? g : 0.0f;
}

__global__ void grad_w1_kernel(const uint8_t *x, uint32_t rows, const float *dpre, float *g) {
    int k = blockIdx.x;
    float acc[F + 1];
    for (int j = 0; j <= F; j++) acc[j] = 0;
    for (uint32_t r = threadIdx.x; r < rows; r += blockDim.x) {
        float d = dpre[(size_t)r * H + k];
        for (int j = 0; j < F; j++) acc[j] = fmaf(d, (float)x[(size_t)r * F + j] * kInScale, acc[j]);
        acc[F] += d;
    }
    // per-warp partial sums, then one fixed-order sum over the warps: the
    // gradient (and so training) does not depend on warp scheduling
    __shared__ float part[8][F + 1];
    for (int j = 0; j <= F; j++) {
        float v = acc[j];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
        if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5][j] = v;
    }
    __syncthreads();
    if (threadIdx.x <= F) {
        float v = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += part[w][threadIdx.x];
        if (threadIdx.x < F)
            g[k * F + threadIdx.x] = v;
        else
            g[H * F + k] = v;
    }
}

__global__ void grad_w2_kernel(uint32_t rows, const float *hid, const float *dout, float *g) {
    int k = blockIdx.x; // H blocks for w2, one more for b2
    float acc = 0;
    for (uint32_t r = threadIdx.x; r < rows; r += blockDim.x) acc += (k < H ? hid[(size_t)r * H + k] : 1.0f) * dout[r];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
    __shared__ float part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float v = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += part[w];
        g[k < H ? H * F + H + k : NW - 1] = v;
    }
}

__global__ void adam_kernel(float *w, const float *g, float *m, float *v, float lr, float wd, float b1t, float b2t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NW) return;
    const float b1 = 0.9f, b2 = 0.999f;
    m[i] = b1 * m[i] + (1 - b1) * g[i];
    v[i] = b2 * v[i] + (1 - b2) * g[i] * g[i];
    float mh = m[i] / (1 - b1t), vh = v[i] / (1 - b2t);
    w[i] -= lr * (mh / (sqrtf(vh) + 1e-8f) + wd * w[i]);
}

struct Buffers {
    float *w = nullptr, *q = nullptr, *scales = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    float *pre = nullptr, *hid = nullptr, *dpre = nullptr, *dout = nullptr, *loss = nullptr;
    uint32_t cap = 0;
    ~Buffers() {
        for (float *p : {w, q, scales, g, m, v, pre, hid, dpre, dout, loss})
            if (p) cudaFree(p);
    }
    bool alloc(uint32_t rows) {
        cap = rows;
        bool ok = cudaMalloc(&w, NW * 4) == cudaSuccess && cudaMalloc(&q, NW * 4) == cudaSuccess &&
                  cudaMalloc(&scales, (H + 1) * 4) == cudaSuccess && cudaMalloc(&g, NW * 4) == cudaSuccess &&
                  cudaMalloc(&m, NW * 4) == cudaSuccess && cudaMalloc(&v, NW * 4) == cudaSuccess &&
                  cudaMalloc(&pre, (size_t)rows * H * 4) == cudaSuccess &&
                  cudaMalloc(&hid, (size_t)rows * H * 4) == cudaSuccess &&
                  cudaMalloc(&dpre, (size_t)rows * H * 4) == cudaSuccess &&
                  cudaMalloc(&dout, (size_t)rows * 4) == cudaSuccess && cudaMalloc(&loss, 4) == cudaSuccess;
        return ok;
    }
};

// quantize + forward + backward of one minibatch; gradients into b.g
void step_grads(Buffers &b, const uint8_t *x, const float *y, uint32_t rows) {
    quantize_kernel<<<1, H>>>(b.w, b.q, b.scales);
    cudaMemset(b.loss, 0, 4);
    forward_kernel<<<(rows + 127) / 128, 128>>>(x, y, rows, b.q, b.pre, b.hid, b.dout, b.loss);
    hidden_grad_kernel<<<(unsigned)(((size_t)rows * H + 255) / 256), 256>>>(rows, b.q, b.pre, b.dout, b.dpre);
    grad_w1_kernel<<<H, 256>>>(x, rows, b.dpre, b.g);
    grad_w2_kernel<<<H + 1, 256>>>(rows, b.hid, b.dout, b.g);
}

} // namespace
} // namespace gpx

using namespace gpx;

extern "C" {

void gpx_train_options_init(gpx_train_options *o) {
    memset(o, 0, sizeof *o);
    o->struct_size = sizeof *o;
    o->epochs = 20;
    o->batch = 8192;
    o->lr = 3e-3f;
    o->weight_decay = 1e-4f;
    o->seed = 7;
}

int gpx_por_grad(int device, const float *w1, const float *b1, const float *w2, float b2, const uint8_t *x,
                 const float *y, uint32_t rows, float *gw1, float *gb1, float *gw2, float *gb2, float *loss) {
    if (!w1 || !b1 || !w2 || !x || !y || !rows || !gw1 || !gb1 || !gw2 || !gb2 || !loss) return GPX_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPX_ERR_NO_GPU;
    if (cudaSetDevice(device) != cudaSuccess) return GPX_ERR_CUDA;
    Buffers b;
    if (!b.alloc(rows)) return GPX_ERR_NOMEM;
    std::vector<float> hw(NW);
    memcpy(hw.data(), w1, H * F * 4);
    memcpy(hw.data() + H * F, b1, H * 4);
    memcpy(hw.data() + H * F + H, w2, H * 4);
    hw[NW - 1] = b2;
    uint8_t *dx = nullptr;
    float *dy = nullptr;
    if (cudaMalloc(&dx, (size_t)rows * F) != cudaSuccess || cudaMalloc(&dy, (size_t)rows * 4) != cudaSuccess) {
        cudaFree(dx);
        return GPX_ERR_NOMEM;
    }
    cudaMemcpy(dx, x, (size_t)rows * F, cudaMemcpyHostToDevice);
    cudaMemcpy(dy, y, (size_t)rows * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(b.w, hw.data(), NW * 4, cudaMemcpyHostToDevice);
    step_grads(b, dx, dy, rows);
    std::vector<float> hg(NW);
    cudaMemcpy(hg.data(), b.g, NW * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(loss, b.loss, 4, cudaMemcpyDeviceToHost);
    cudaError_t e = cudaGetLastError();
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return GPX_ERR_CUDA;
    memcpy(gw1, hg.data(), H * F * 4);
    memcpy(gb1, hg.data() + H * F, H * 4);
    memcpy(gw2, hg.data() + H * F + H, H * 4);
    *gb2 = hg[NW - 1];
    return GPX_OK;
}

int gpx_por_train(const uint8_t *x, const float *y, uint64_t rows, const gpx_train_options *o, gpx_por_model *out,
                  float *final_loss) {
    if (!x || !y || !rows || !o || !out || o->struct_size != sizeof(gpx_train_options) || rows > (1ull << 31))
        return GPX_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return GPX_ERR_NO_GPU;
    if (cudaSetDevice(o->device) != cudaSuccess) return GPX_ERR_CUDA;
    const uint32_t bs = std::max<uint32_t>(256, std::min<uint32_t>(o->batch ? o->batch : 8192, (uint32_t)rows));
    Buffers b;
    if (!b.alloc(bs)) return GPX_ERR_NOMEM;
    // initial weights: uniform(+-1/sqrt(fan_in)), seeded
    std::mt19937_64 rng(o->seed);
    std::vector<float> hw(NW, 0.0f);
    std::uniform_real_distribution<float> u1(-1.0f / std::sqrt((float)F), 1.0f / std::sqrt((float)F));
    std::uniform_real_distribution<float> u2(-1.0f / std::sqrt((float)H), 1.0f / std::sqrt((float)H));
    for (int i = 0; i < H * F; i++) hw[i] = u1(rng);
    for (int i = 0; i < H; i++) hw[H * F + H + i] = u2(rng);
    // rows in a seeded random order, uploaded once
    std::vector<uint64_t> perm(rows);
    for (uint64_t i = 0; i < rows; i++) perm[i] = i;
    std::shuffle(perm.begin(), perm.end(), rng);
    std::vector<uint8_t> hx((size_t)rows * F);
    std::vector<float> hy(rows);
    for (uint64_t i = 0; i < rows; i++) {
        memcpy(&hx[i * F], x + perm[i] * F, F);
        hy[i] = y[perm[i]];
    }
    uint8_t *dx = nullptr;
    float *dy = nullptr;
    if (cudaMalloc(&dx, hx.size()) != cudaSuccess || cudaMalloc(&dy, rows * 4) != cudaSuccess) {
        cudaFree(dx);
        return GPX_ERR_NOMEM;
    }
    cudaMemcpy(dx, hx.data(), hx.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(dy, hy.data(), rows * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(b.w, hw.data(), NW * 4, cudaMemcpyHostToDevice);
    cudaMemset(b.m, 0, NW * 4);
    cudaMemset(b.v, 0, NW * 4);
    float b1t = 1.0f, b2t = 1.0f, last = 0.0f;
    uint64_t steps = 0;
    for (uint32_t ep = 0; ep < (o->epochs ? o->epochs : 20); ep++) {
        double ep_loss = 0;
        uint64_t nb = 0;
        for (uint64_t r0 = 0; r0 + bs <= rows || (r0 == 0 && rows < bs); r0 += bs) {
            uint32_t n = (uint32_t)std::min<uint64_t>(bs, rows - r0);
            step_grads(b, dx + r0 * F, dy + r0, n);
            b1t *= 0.9f;
            b2t *= 0.999f;
            adam_kernel<<<(NW + 255) / 256, 256>>>(b.w, b.g, b.m, b.v, o->lr, o->weight_decay, b1t, b2t);
            float l = 0;
            cudaMemcpy(&l, b.loss, 4, cudaMemcpyDeviceToHost);
            ep_loss += l;
            nb++;
            steps++;
            if (rows < bs) break;
        }
        last = (float)(ep_loss / std::max<uint64_t>(nb, 1));
    }
    // export: int8 weights, per-row scales with the input scale folded in
    quantize_kernel<<<1, H>>>(b.w, b.q, b.scales);
    std::vector<float> hq(NW), hs(H + 1);
    cudaMemcpy(hw.data(), b.w, NW * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(hs.data(), b.scales, (H + 1) * 4, cudaMemcpyDeviceToHost);
    cudaError_t e = cudaGetLastError();
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return GPX_ERR_CUDA;
    memset(out, 0, sizeof *out);
    for (int k = 0; k < H; k++) {
        for (int j = 0; j < F; j++)
            out->w1[k][j] =
                (int8_t)std::lrint(std::min(127.0f, std::max(-127.0f, hw[k * F + j] / hs[k])));
        out->s1[k] = hs[k] * kInScale;
        out->b1[k] = hw[H * F + k];
        out->w2[k] = (int8_t)std::lrint(std::min(127.0f, std::max(-127.0f, hw[H * F + H + k] / hs[H])));
    }
    out->s2 = hs[H];
    out->b2 = hw[NW - 1];
    if (final_loss) *final_loss = last;
    (void)steps;
    return GPX_OK;
}

} // extern "C"
