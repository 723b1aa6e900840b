// Block cost model: MLP 6 -> 64 -> 64 -> 2 (ReLU, FP32) — inference,
// loss/gradient and Adam training on the device.
//
// It replaces the reference's pickled RandomForest (models/
// density_threshold_spmv.pkl, queried per block at
// utils/convert_real_to_vbr.py:58): instead of a dense/sparse class it
// predicts log2 of the device time of both forms of a block, so the choice is
// argmin and the margin is a time.
//
// Input features (one row of 6 floats per block): rows, cols, nnz, density,
// variance of nnz per row, SpMM width N.  In-kernel transform:
//   g_i = log2(1 + f_i) for i != 3, g_3 = f_3 (density),
//   z_i = (g_i - mean_i) / std_i   (mean/std set with sable_mlp_set_norm).
// Parameters, flat, row-major (out x in):
//   W1[64][6] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]   = 4738 floats.
//
// Kernels
//   infer   one thread per block: layer 1 into 64 registers, layer 2 one
//           neuron at a time folded straight into the 2 outputs.  Parameters
//           sit in shared memory; every warp reads the same word (broadcast).
//   grad    128 samples per CTA.  Phase 1, one thread per sample: forward,
//           output error, back-propagation to dZ2 and dZ1; the activations
//           and errors go to shared memory as [feature][sample] with a row
//           stride of 129 floats (bank-conflict-free for both phases).
//           Phase 2, all threads over the 4738 parameters: each gradient
//           entry is a dot product over the CTA's samples, written to a
//           per-CTA partial row.
//   reduce  one thread per parameter sums the partial rows in CTA order
//           (deterministic, no atomics), then writes the gradient or applies
//           one Adam step.
// Loss: L = 1/(2n) sum_samples sum_outputs (o - t)^2, so dL/do = (o - t)/n.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "sable.h"
#include "sable_internal.h"
#include "plan_internal.h"

namespace {

constexpr int NF = 6, H1N = 64, H2N = 64, NO = 2;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H1N * NF, OFF_W2 = OFF_B1 + H1N, OFF_B2 = OFF_W2 + H2N * H1N,
              OFF_W3 = OFF_B2 + H2N, OFF_B3 = OFF_W3 + NO * H2N, NP = OFF_B3 + NO;
static_assert(NP == SABLE_MLP_NPARAMS, "parameter count");
constexpr int BS = 128;          // samples per CTA in the gradient kernel
constexpr int SP = BS + 1;       // row stride of [feature][sample] arrays
constexpr int INFER_THREADS = 128;

struct GradSmem {
    static constexpr int PAR = 0;                      // params + norm (NP + 12)
    static constexpr int X = PAR + NP + 12;            // [NF][SP]
    static constexpr int H1 = X + NF * SP;             // [64][SP]
    static constexpr int H2 = H1 + H1N * SP;           // [64][SP]
    static constexpr int DZ2 = H2 + H2N * SP;          // [64][SP]
    static constexpr int DZ1 = DZ2 + H2N * SP;         // [64][SP]
    static constexpr int DO = DZ1 + H1N * SP;          // [2][SP]
    static constexpr int RED = DO + NO * SP;           // [BS] loss reduction
    static constexpr int TOTAL = RED + BS;             // floats
};

__device__ __forceinline__ void load_params(float *sp, const float *__restrict__ params, const float *__restrict__ norm) {
    for (int i = threadIdx.x; i < NP; i += blockDim.x) sp[i] = params[i];
    for (int i = threadIdx.x; i < 12; i += blockDim.x) sp[NP + i] = norm[i];
}

__device__ __forceinline__ void features(const float *__restrict__ f, const float *sp, float (&x)[NF]) {
#pragma unroll
    for (int i = 0; i < NF; ++i) {
        const float v = f[i];
        const float g = i == 3 ? v : log2f(1.0f + v);
        x[i] = (g - sp[NP + i]) / sp[NP + 6 + i];
    }
}

__global__ void __launch_bounds__(INFER_THREADS)
mlp_infer_kernel(const float *__restrict__ params, const float *__restrict__ norm, const float *__restrict__ feat,
                 int n, float *__restrict__ out) {
    __shared__ float sp[NP + 12];
    load_params(sp, params, norm);
    __syncthreads();
    const int s = blockIdx.x * INFER_THREADS + threadIdx.x;
    if (s >= n) return;
    float x[NF];
    features(feat + (int64_t)s * NF, sp, x);
    float h1[H1N];
#pragma unroll
    for (int k = 0; k < H1N; ++k) {
        float z = sp[OFF_B1 + k];
#pragma unroll
        for (int i = 0; i < NF; ++i) z = fmaf(sp[OFF_W1 + k * NF + i], x[i], z);
        h1[k] = fmaxf(z, 0.f);
    }
    float o0 = sp[OFF_B3], o1 = sp[OFF_B3 + 1];
    for (int j = 0; j < H2N; ++j) {
        float z = sp[OFF_B2 + j];
#pragma unroll
        for (int k = 0; k < H1N; ++k) z = fmaf(sp[OFF_W2 + j * H1N + k], h1[k], z);
        z = fmaxf(z, 0.f);
        o0 = fmaf(sp[OFF_W3 + j], z, o0);
        o1 = fmaf(sp[OFF_W3 + H2N + j], z, o1);
    }
    out[2 * (int64_t)s] = o0;
    out[2 * (int64_t)s + 1] = o1;
}

// idx (optional): sample s of the batch is row idx[s] of feat / target.
__global__ void __launch_bounds__(BS)
mlp_grad_kernel(const float *__restrict__ params, const float *__restrict__ norm, const float *__restrict__ feat,
                const float *__restrict__ target, const int32_t *__restrict__ idx, int n, float inv_n,
                float *__restrict__ partial, float *__restrict__ loss_partial) {
    extern __shared__ float sm[];
    using L = GradSmem;
    float *sp = sm + L::PAR;
    float *Xs = sm + L::X, *H1s = sm + L::H1, *H2s = sm + L::H2, *DZ2s = sm + L::DZ2, *DZ1s = sm + L::DZ1;
    float *DOs = sm + L::DO, *red = sm + L::RED;
    load_params(sp, params, norm);
    __syncthreads();

    // ---- phase 1: one thread per sample --------------------------------------
    const int s = threadIdx.x;
    const int gs = blockIdx.x * BS + s;
    float lsum = 0.f;
    if (gs < n) {
        const int64_t row = idx ? (int64_t)idx[gs] : (int64_t)gs;
        float x[NF];
        features(feat + row * NF, sp, x);
#pragma unroll
        for (int i = 0; i < NF; ++i) Xs[i * SP + s] = x[i];
        float h1[H1N];
#pragma unroll
        for (int k = 0; k < H1N; ++k) {
            float z = sp[OFF_B1 + k];
#pragma unroll
            for (int i = 0; i < NF; ++i) z = fmaf(sp[OFF_W1 + k * NF + i], x[i], z);
            h1[k] = fmaxf(z, 0.f);
            H1s[k * SP + s] = h1[k];
        }
        float o0 = sp[OFF_B3], o1 = sp[OFF_B3 + 1];
        for (int j = 0; j < H2N; ++j) {
            float z = sp[OFF_B2 + j];
#pragma unroll
            for (int k = 0; k < H1N; ++k) z = fmaf(sp[OFF_W2 + j * H1N + k], h1[k], z);
            z = fmaxf(z, 0.f);
            H2s[j * SP + s] = z;
            o0 = fmaf(sp[OFF_W3 + j], z, o0);
            o1 = fmaf(sp[OFF_W3 + H2N + j], z, o1);
        }
        const float e0 = o0 - target[2 * row], e1 = o1 - target[2 * row + 1];
        lsum = e0 * e0 + e1 * e1;
        const float d0 = e0 * inv_n, d1 = e1 * inv_n;
        DOs[s] = d0;
        DOs[SP + s] = d1;
        float dh1[H1N];
#pragma unroll
        for (int k = 0; k < H1N; ++k) dh1[k] = 0.f;
        for (int j = 0; j < H2N; ++j) {
            const float g = H2s[j * SP + s] > 0.f ? fmaf(d0, sp[OFF_W3 + j], d1 * sp[OFF_W3 + H2N + j]) : 0.f;
            DZ2s[j * SP + s] = g;
#pragma unroll
            for (int k = 0; k < H1N; ++k) dh1[k] = fmaf(g, sp[OFF_W2 + j * H1N + k], dh1[k]);
        }
#pragma unroll
        for (int k = 0; k < H1N; ++k) DZ1s[k * SP + s] = h1[k] > 0.f ? dh1[k] : 0.f;
    } else {
        // an absent sample contributes nothing to any sum
#pragma unroll
        for (int i = 0; i < NF; ++i) Xs[i * SP + s] = 0.f;
        for (int k = 0; k < H1N; ++k) {
            H1s[k * SP + s] = 0.f;
            DZ1s[k * SP + s] = 0.f;
        }
        for (int j = 0; j < H2N; ++j) {
            H2s[j * SP + s] = 0.f;
            DZ2s[j * SP + s] = 0.f;
        }
        DOs[s] = 0.f;
        DOs[SP + s] = 0.f;
    }
    red[s] = lsum;
    __syncthreads();

    // ---- phase 2: gradient entries, each a dot product over the CTA's samples
    const int cnt = min(BS, n - blockIdx.x * BS);
    float *P = partial + (int64_t)blockIdx.x * NP;
    for (int p = threadIdx.x; p < NP; p += BS) {
        const float *u, *v = nullptr;
        if (p < OFF_B1) {
            u = DZ1s + (p / NF) * SP;
            v = Xs + (p % NF) * SP;
        } else if (p < OFF_W2) {
            u = DZ1s + (p - OFF_B1) * SP;
        } else if (p < OFF_B2) {
            const int q = p - OFF_W2;
            u = DZ2s + (q / H1N) * SP;
            v = H1s + (q % H1N) * SP;
        } else if (p < OFF_W3) {
            u = DZ2s + (p - OFF_B2) * SP;
        } else if (p < OFF_B3) {
            const int q = p - OFF_W3;
            u = DOs + (q / H2N) * SP;
            v = H2s + (q % H2N) * SP;
        } else {
            u = DOs + (p - OFF_B3) * SP;
        }
        float acc = 0.f;
        if (v) {
            for (int t = 0; t < cnt; ++t) acc = fmaf(u[t], v[t], acc);
        } else {
            for (int t = 0; t < cnt; ++t) acc += u[t];
        }
        P[p] = acc;
    }
    // loss: fixed-shape tree over the CTA's samples
    for (int w = BS / 2; w > 0; w >>= 1) {
        if (s < w) red[s] += red[s + w];
        __syncthreads();
    }
    if (s == 0) loss_partial[blockIdx.x] = red[0] * 0.5f * inv_n;
}

// mode 0: grad[p] = sum of partials;  mode 1: Adam step on params.
__global__ void mlp_reduce_kernel(const float *__restrict__ partial, const float *__restrict__ loss_partial, int nblk,
                                  int mode, float *__restrict__ grad, float *__restrict__ params, float *__restrict__ m1,
                                  float *__restrict__ m2, float lr, float beta1, float beta2, float eps, float c1,
                                  float c2, float *__restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0 && loss) {
        float l = 0.f;
        for (int b = 0; b < nblk; ++b) l += loss_partial[b];
        *loss = l;
    }
    if (p >= NP) return;
    float g = 0.f;
    for (int b = 0; b < nblk; ++b) g += partial[(int64_t)b * NP + p];
    if (mode == 0) {
        grad[p] = g;
        return;
    }
    const float a = beta1 * m1[p] + (1.f - beta1) * g;
    const float b = beta2 * m2[p] + (1.f - beta2) * g * g;
    m1[p] = a;
    m2[p] = b;
    // c1 = 1 / (1 - beta1^t), c2 = 1 / (1 - beta2^t)
    params[p] -= lr * (a * c1) / (sqrtf(b * c2) + eps);
}

}  // namespace

struct sable_mlp {
    int device = 0;
    float *d_params = nullptr, *d_norm = nullptr, *d_m1 = nullptr, *d_m2 = nullptr;
    float *d_partial = nullptr, *d_loss_partial = nullptr;
    int64_t partial_blocks = 0;
    int64_t step = 0;
};

using namespace sable;

namespace {

int ensure_partial(sable_mlp *m, int64_t nblk) {
    if (nblk <= m->partial_blocks) return SABLE_OK;
    cudaFree(m->d_partial);
    cudaFree(m->d_loss_partial);
    m->d_partial = m->d_loss_partial = nullptr;
    m->partial_blocks = 0;
    cudaError_t e = cudaMalloc(&m->d_partial, (size_t)nblk * NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->d_loss_partial, (size_t)nblk * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(e, "mlp gradient scratch");
    m->partial_blocks = nblk;
    return SABLE_OK;
}

int run_grad(sable_mlp *m, const float *feat, const float *target, const int32_t *idx, int32_t n, cudaStream_t st) {
    const int64_t nblk = (n + BS - 1) / BS;
    int rc = ensure_partial(m, nblk);
    if (rc) return rc;
    const int smem = GradSmem::TOTAL * (int)sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return cuda_fail(e, "mlp grad smem attribute");
    mlp_grad_kernel<<<(unsigned)nblk, BS, smem, st>>>(m->d_params, m->d_norm, feat, target, idx, n, 1.0f / (float)n,
                                                      m->d_partial, m->d_loss_partial);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mlp grad launch");
    return SABLE_OK;
}

}  // namespace

extern "C" {

int sable_mlp_create(sable_mlp **out) {
    if (!out) return fail(SABLE_ERR_ARG, "null argument");
    *out = nullptr;
    sable_mlp *m = new (std::nothrow) sable_mlp();
    if (!m) return fail(SABLE_ERR_NOMEM, "host allocation");
    cudaGetDevice(&m->device);
    cudaError_t e = cudaMalloc(&m->d_params, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->d_norm, 12 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->d_m1, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->d_m2, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->d_params, 0, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->d_m1, 0, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->d_m2, 0, NP * sizeof(float));
    if (e == cudaSuccess) {
        float norm[12];
        for (int i = 0; i < 6; ++i) norm[i] = 0.f, norm[6 + i] = 1.f;
        e = cudaMemcpy(m->d_norm, norm, sizeof norm, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        sable_mlp_destroy(m);
        return cuda_fail(e, "mlp allocation");
    }
    *out = m;
    return SABLE_OK;
}

int sable_mlp_destroy(sable_mlp *m) {
    if (!m) return SABLE_OK;
    set_device(m->device);
    cudaFree(m->d_params);
    cudaFree(m->d_norm);
    cudaFree(m->d_m1);
    cudaFree(m->d_m2);
    cudaFree(m->d_partial);
    cudaFree(m->d_loss_partial);
    delete m;
    return SABLE_OK;
}

// Also resets the Adam state (moments and step count).
int sable_mlp_set_params(sable_mlp *m, const float *params_host) {
    if (!m || !params_host) return fail(SABLE_ERR_ARG, "null argument");
    int rc = set_device(m->device);
    if (rc) return rc;
    cudaError_t e = cudaMemcpy(m->d_params, params_host, NP * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->d_m1, 0, NP * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->d_m2, 0, NP * sizeof(float));
    if (e != cudaSuccess) return cuda_fail(e, "mlp set params");
    m->step = 0;
    return SABLE_OK;
}

int sable_mlp_get_params(const sable_mlp *m, float *params_host) {
    if (!m || !params_host) return fail(SABLE_ERR_ARG, "null argument");
    int rc = set_device(m->device);
    if (rc) return rc;
    cudaError_t e = cudaMemcpy(params_host, m->d_params, NP * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "mlp get params");
    return SABLE_OK;
}

int sable_mlp_set_norm(sable_mlp *m, const float *mean6, const float *std6) {
    if (!m || !mean6 || !std6) return fail(SABLE_ERR_ARG, "null argument");
    float norm[12];
    for (int i = 0; i < 6; ++i) {
        if (!(std6[i] > 0.f)) return fail(SABLE_ERR_ARG, "feature %d: std must be > 0", i);
        norm[i] = mean6[i];
        norm[6 + i] = std6[i];
    }
    int rc = set_device(m->device);
    if (rc) return rc;
    cudaError_t e = cudaMemcpy(m->d_norm, norm, sizeof norm, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "mlp set norm");
    return SABLE_OK;
}

int sable_mlp_infer(sable_mlp *m, const float *feat_dev, int32_t n, float *out_dev, void *stream) {
    if (!m || n < 0 || (n > 0 && (!feat_dev || !out_dev))) return fail(SABLE_ERR_ARG, "bad argument");
    if (n == 0) return SABLE_OK;
    int rc = set_device(m->device);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    mlp_infer_kernel<<<(n + INFER_THREADS - 1) / INFER_THREADS, INFER_THREADS, 0, st>>>(m->d_params, m->d_norm,
                                                                                       feat_dev, n, out_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mlp infer launch");
    return SABLE_OK;
}

int sable_mlp_loss_grad(sable_mlp *m, const float *feat_dev, const float *target_dev, int32_t n, float *grad_dev,
                        float *loss_dev, void *stream) {
    if (!m || n <= 0 || !feat_dev || !target_dev || !grad_dev) return fail(SABLE_ERR_ARG, "bad argument");
    int rc = set_device(m->device);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rc = run_grad(m, feat_dev, target_dev, nullptr, n, st);
    if (rc) return rc;
    const int nblk = (n + BS - 1) / BS;
    mlp_reduce_kernel<<<(NP + 255) / 256, 256, 0, st>>>(m->d_partial, m->d_loss_partial, nblk, 0, grad_dev, nullptr,
                                                        nullptr, nullptr, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, loss_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mlp reduce launch");
    return SABLE_OK;
}

int sable_mlp_train_step(sable_mlp *m, const float *feat_dev, const float *target_dev, const int32_t *idx_dev,
                         int32_t n, float lr, float *loss_dev, void *stream) {
    if (!m || n <= 0 || !feat_dev || !target_dev || !(lr > 0.f)) return fail(SABLE_ERR_ARG, "bad argument");
    int rc = set_device(m->device);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rc = run_grad(m, feat_dev, target_dev, idx_dev, n, st);
    if (rc) return rc;
    const int nblk = (n + BS - 1) / BS;
    m->step += 1;
    const double b1 = 0.9, b2 = 0.999;
    const float c1 = (float)(1.0 / (1.0 - pow(b1, (double)m->step)));
    const float c2 = (float)(1.0 / (1.0 - pow(b2, (double)m->step)));
    mlp_reduce_kernel<<<(NP + 255) / 256, 256, 0, st>>>(m->d_partial, m->d_loss_partial, nblk, 1, nullptr, m->d_params,
                                                        m->d_m1, m->d_m2, lr, (float)b1, (float)b2, 1e-8f, c1, c2,
                                                        loss_dev);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mlp adam launch");
    return SABLE_OK;
}

}  // extern "C"
