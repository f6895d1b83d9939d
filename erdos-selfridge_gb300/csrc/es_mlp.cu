// Learned cost model of the planner: a 3-layer FP32 MLP (in -> H -> H -> out, ReLU), trained and
// evaluated on the GPU by these kernels.  Sizes are tiny (in <= 64, H <= 64, out <= 8, samples
// in the thousands), so the kernels are plain SIMT FP32 with weights and one sample tile staged in
// shared memory; tensor cores would not pay for themselves at this size.
//
// Parameters, flat FP32: W1[H][D], b1[H], W2[H][H], b2[H], W3[O][H], b3[O].
// Loss: mean squared error over samples x outputs.  Gradients are reduced deterministically:
// each CTA writes the partial gradient of its sample tile, one kernel sums the tiles in order.
// Optimiser: Adam (Kingma & Ba), bias-corrected.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/es_gb300.h"

namespace {

constexpr int kTile = 32;        // samples per CTA
constexpr int kMaxD = 64, kMaxH = 64, kMaxO = 8;   // keeps a tile's shared memory under 48 KB

thread_local std::string g_mlp_err;
int mlp_fail(int code, const std::string& m) {
    g_mlp_err = m;
    return code;
}

struct Dims {
    int D, H, O;
    __host__ __device__ int nW1() const { return H * D; }
    __host__ __device__ int oB1() const { return nW1(); }
    __host__ __device__ int oW2() const { return oB1() + H; }
    __host__ __device__ int oB2() const { return oW2() + H * H; }
    __host__ __device__ int oW3() const { return oB2() + H; }
    __host__ __device__ int oB3() const { return oW3() + O * H; }
    __host__ __device__ int n() const { return oB3() + O; }
};

// Forward of one tile; optionally keeps activations for the backward pass.
// blockDim.x = H (>= O).  smem: x[T][D], a1[T][H], a2[T][H].
__global__ void mlp_forward_kernel(Dims d, const float* __restrict__ P, const float* __restrict__ X,
                                   uint64_t n, float* __restrict__ Y) {
    extern __shared__ float sm[];
    float* xs = sm;
    float* a1 = xs + kTile * d.D;
    float* a2 = a1 + kTile * d.H;
    const uint64_t n0 = (uint64_t)blockIdx.x * kTile;
    const int j = threadIdx.x;
    for (int i = threadIdx.x; i < kTile * d.D; i += blockDim.x) {
        const uint64_t s = n0 + i / d.D;
        xs[i] = s < n ? X[s * d.D + i % d.D] : 0.f;
    }
    __syncthreads();
    if (j < d.H) {
        const float* w = P + j * d.D;
        const float b = P[d.oB1() + j];
        for (int t = 0; t < kTile; ++t) {
            float acc = b;
            for (int i = 0; i < d.D; ++i) acc = fmaf(w[i], xs[t * d.D + i], acc);
            a1[t * d.H + j] = fmaxf(acc, 0.f);
        }
    }
    __syncthreads();
    if (j < d.H) {
        const float* w = P + d.oW2() + j * d.H;
        const float b = P[d.oB2() + j];
        for (int t = 0; t < kTile; ++t) {
            float acc = b;
            for (int i = 0; i < d.H; ++i) acc = fmaf(w[i], a1[t * d.H + i], acc);
            a2[t * d.H + j] = fmaxf(acc, 0.f);
        }
    }
    __syncthreads();
    if (j < d.O) {
        const float* w = P + d.oW3() + j * d.H;
        const float b = P[d.oB3() + j];
        for (int t = 0; t < kTile; ++t) {
            const uint64_t s = n0 + t;
            if (s >= n) break;
            float acc = b;
            for (int i = 0; i < d.H; ++i) acc = fmaf(w[i], a2[t * d.H + i], acc);
            Y[s * d.O + j] = acc;
        }
    }
}

// Forward + backward of one tile; writes this tile's gradient (sum over its samples of
// d(loss)/d(params), with loss = sum (y - t)^2 / (n * O)) to G[blockIdx.x][n_params] and the
// tile's squared error to L[blockIdx.x].  blockDim.x = H.
__global__ void mlp_grad_kernel(Dims d, const float* __restrict__ P, const float* __restrict__ X,
                                const float* __restrict__ T, const uint32_t* __restrict__ idx,
                                uint64_t n, float scale, float* __restrict__ G, float* __restrict__ L) {
    extern __shared__ float sm[];
    float* xs = sm;                       // [T][D]
    float* a1 = xs + kTile * d.D;         // [T][H]
    float* a2 = a1 + kTile * d.H;         // [T][H]
    float* go = a2 + kTile * d.H;         // [T][O]   d loss / d out
    float* g2 = go + kTile * kMaxO;       // [T][H]   d loss / d a2 (pre-activation masked)
    float* g1 = g2 + kTile * d.H;         // [T][H]
    float* red = g1 + kTile * d.H;        // [H]
    const uint64_t n0 = (uint64_t)blockIdx.x * kTile;
    const int j = threadIdx.x;
    const int nt = (int)((n - n0) < (uint64_t)kTile ? (n - n0) : (uint64_t)kTile);
    for (int i = threadIdx.x; i < kTile * d.D; i += blockDim.x) {
        const int t = i / d.D;
        const uint64_t s = n0 + t;
        xs[i] = t < nt ? X[(uint64_t)(idx ? idx[s] : s) * d.D + i % d.D] : 0.f;
    }
    __syncthreads();
    // forward
    {
        const float* w = P + j * d.D;
        const float b = P[d.oB1() + j];
        for (int t = 0; t < kTile; ++t) {
            float acc = b;
            for (int i = 0; i < d.D; ++i) acc = fmaf(w[i], xs[t * d.D + i], acc);
            a1[t * d.H + j] = fmaxf(acc, 0.f);
        }
    }
    __syncthreads();
    {
        const float* w = P + d.oW2() + j * d.H;
        const float b = P[d.oB2() + j];
        for (int t = 0; t < kTile; ++t) {
            float acc = b;
            for (int i = 0; i < d.H; ++i) acc = fmaf(w[i], a1[t * d.H + i], acc);
            a2[t * d.H + j] = fmaxf(acc, 0.f);
        }
    }
    __syncthreads();
    float sq = 0.f;
    if (j < d.O) {
        const float* w = P + d.oW3() + j * d.H;
        const float b = P[d.oB3() + j];
        for (int t = 0; t < kTile; ++t) {
            float e = 0.f;
            if (t < nt) {
                float acc = b;
                for (int i = 0; i < d.H; ++i) acc = fmaf(w[i], a2[t * d.H + i], acc);
                const uint64_t s = n0 + t;
                e = acc - T[(uint64_t)(idx ? idx[s] : s) * d.O + j];
                sq += e * e;
            }
            go[t * kMaxO + j] = 2.f * e * scale;
        }
    }
    red[j] = sq;
    __syncthreads();
    // back through layer 3: g2 = (W3^T go) * [a2 > 0]
    for (int t = 0; t < kTile; ++t) {
        float acc = 0.f;
        for (int o = 0; o < d.O; ++o) acc = fmaf(P[d.oW3() + o * d.H + j], go[t * kMaxO + o], acc);
        g2[t * d.H + j] = a2[t * d.H + j] > 0.f ? acc : 0.f;
    }
    __syncthreads();
    // g1 = (W2^T g2) * [a1 > 0]
    for (int t = 0; t < kTile; ++t) {
        float acc = 0.f;
        for (int i = 0; i < d.H; ++i) acc = fmaf(P[d.oW2() + i * d.H + j], g2[t * d.H + i], acc);
        g1[t * d.H + j] = a1[t * d.H + j] > 0.f ? acc : 0.f;
    }
    __syncthreads();
    float* g = G + (uint64_t)blockIdx.x * d.n();
    // dW1[j][:], db1[j]
    for (int i = 0; i < d.D; ++i) {
        float acc = 0.f;
        for (int t = 0; t < kTile; ++t) acc = fmaf(g1[t * d.H + j], xs[t * d.D + i], acc);
        g[j * d.D + i] = acc;
    }
    {
        float acc = 0.f;
        for (int t = 0; t < kTile; ++t) acc += g1[t * d.H + j];
        g[d.oB1() + j] = acc;
    }
    // dW2[j][:], db2[j]
    for (int i = 0; i < d.H; ++i) {
        float acc = 0.f;
        for (int t = 0; t < kTile; ++t) acc = fmaf(g2[t * d.H + j], a1[t * d.H + i], acc);
        g[d.oW2() + j * d.H + i] = acc;
    }
    {
        float acc = 0.f;
        for (int t = 0; t < kTile; ++t) acc += g2[t * d.H + j];
        g[d.oB2() + j] = acc;
    }
    // dW3[o][j], db3[o]
    for (int o = 0; o < d.O; ++o) {
        float acc = 0.f;
        for (int t = 0; t < kTile; ++t) acc = fmaf(go[t * kMaxO + o], a2[t * d.H + j], acc);
        g[d.oW3() + o * d.H + j] = acc;
    }
    if (j < d.O) {
        float acc = 0.f;
        for (int t = 0; t < kTile; ++t) acc += go[t * kMaxO + j];
        g[d.oB3() + j] = acc;
    }
    __syncthreads();
    if (j == 0) {
        float s = 0.f;
        for (int i = 0; i < d.H; ++i) s += red[i];
        L[blockIdx.x] = s;
    }
}

// Deterministic sum of the tiles' partial gradients (and losses) in tile order.
__global__ void mlp_reduce_kernel(const float* __restrict__ G, int tiles, int np, float* __restrict__ out,
                                  const float* __restrict__ L, float* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np) {
        float acc = 0.f;
        for (int t = 0; t < tiles; ++t) acc += G[(uint64_t)t * np + p];
        out[p] = acc;
    }
    if (p == 0 && loss) {
        float s = 0.f;
        for (int t = 0; t < tiles; ++t) s += L[t];
        *loss = s;
    }
}

__global__ void mlp_adam_kernel(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, int np, float lr, float b1, float b2, float eps,
                                float c1, float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const float gi = g[p];
    const float mi = b1 * m[p] + (1.f - b1) * gi;
    const float vi = b2 * v[p] + (1.f - b2) * gi * gi;
    m[p] = mi;
    v[p] = vi;
    P[p] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

size_t fwd_smem(const Dims& d) { return sizeof(float) * (size_t)kTile * (d.D + 2 * d.H); }
size_t grad_smem(const Dims& d) {
    return sizeof(float) * ((size_t)kTile * (d.D + 4 * d.H + kMaxO) + d.H);
}

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

}  // namespace

struct es_mlp {
    Dims d{};
    float* P = nullptr;      // parameters
    float* m = nullptr;      // Adam moments
    float* v = nullptr;
    float* g = nullptr;      // reduced gradient
    float* loss = nullptr;   // device scalar
    uint64_t steps = 0;
};

extern "C" {

const char* es_mlp_last_error(void) { return g_mlp_err.c_str(); }

int es_mlp_create(uint32_t in_dim, uint32_t hidden, uint32_t out_dim, uint64_t seed, es_mlp** out) {
    if (!out) return mlp_fail(ES_ERR_ARG, "null output");
    *out = nullptr;
    if (in_dim < 1 || in_dim > kMaxD || hidden < 8 || hidden > kMaxH || hidden % 32 || out_dim < 1 ||
        out_dim > kMaxO || out_dim > hidden)
        return mlp_fail(ES_ERR_RANGE, "MLP dims must be in <= 64, hidden 32 or 64, out <= 8");
    es_mlp* M = new es_mlp();
    M->d = Dims{(int)in_dim, (int)hidden, (int)out_dim};
    const int np = M->d.n();
    std::vector<float> h(np, 0.f);
    // He-uniform init for the ReLU layers, Glorot-uniform for the output, zero biases
    uint64_t s = seed;
    auto uni = [&](float a) { return (float)(((splitmix(s) >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0) * a; };
    for (int i = 0; i < M->d.nW1(); ++i) h[i] = uni(std::sqrt(6.f / in_dim));
    for (int i = 0; i < hidden * hidden; ++i) h[M->d.oW2() + i] = uni(std::sqrt(6.f / hidden));
    for (int i = 0; i < (int)out_dim * (int)hidden; ++i) h[M->d.oW3() + i] = uni(std::sqrt(6.f / (hidden + out_dim)));
    cudaError_t e = cudaMalloc(&M->P, 4ull * np);
    if (e == cudaSuccess) e = cudaMalloc(&M->m, 4ull * np);
    if (e == cudaSuccess) e = cudaMalloc(&M->v, 4ull * np);
    if (e == cudaSuccess) e = cudaMalloc(&M->g, 4ull * np);
    if (e == cudaSuccess) e = cudaMalloc(&M->loss, 4);
    if (e == cudaSuccess) e = cudaMemcpy(M->P, h.data(), 4ull * np, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(M->m, 0, 4ull * np);
    if (e == cudaSuccess) e = cudaMemset(M->v, 0, 4ull * np);
    if (e != cudaSuccess) {
        cudaFree(M->P); cudaFree(M->m); cudaFree(M->v); cudaFree(M->g); cudaFree(M->loss);
        delete M;
        return mlp_fail(ES_ERR_CUDA, std::string("MLP setup: ") + cudaGetErrorString(e));
    }
    *out = M;
    return ES_OK;
}

int es_mlp_destroy(es_mlp* M) {
    if (!M) return ES_OK;
    cudaFree(M->P); cudaFree(M->m); cudaFree(M->v); cudaFree(M->g); cudaFree(M->loss);
    delete M;
    return ES_OK;
}

int es_mlp_num_params(const es_mlp* M, uint64_t* n) {
    if (!M || !n) return mlp_fail(ES_ERR_ARG, "null argument");
    *n = (uint64_t)M->d.n();
    return ES_OK;
}

int es_mlp_get_params(es_mlp* M, float* out, uint64_t n) {
    if (!M || !out || n != (uint64_t)M->d.n()) return mlp_fail(ES_ERR_ARG, "bad parameter buffer");
    cudaError_t e = cudaMemcpy(out, M->P, 4ull * n, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? ES_OK : mlp_fail(ES_ERR_CUDA, cudaGetErrorString(e));
}

int es_mlp_set_params(es_mlp* M, const float* in, uint64_t n) {
    if (!M || !in || n != (uint64_t)M->d.n()) return mlp_fail(ES_ERR_ARG, "bad parameter buffer");
    cudaError_t e = cudaMemcpy(M->P, in, 4ull * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(M->m, 0, 4ull * n);
    if (e == cudaSuccess) e = cudaMemset(M->v, 0, 4ull * n);
    M->steps = 0;
    return e == cudaSuccess ? ES_OK : mlp_fail(ES_ERR_CUDA, cudaGetErrorString(e));
}

// Y[n][O] = MLP(X[n][D]); host buffers.
int es_mlp_forward(es_mlp* M, const float* X, uint64_t n, float* Y) {
    if (!M || (n && (!X || !Y))) return mlp_fail(ES_ERR_ARG, "null argument");
    if (n == 0) return ES_OK;
    const Dims d = M->d;
    float *dx = nullptr, *dy = nullptr;
    cudaError_t e = cudaMalloc(&dx, 4ull * n * d.D);
    if (e == cudaSuccess) e = cudaMalloc(&dy, 4ull * n * d.O);
    if (e == cudaSuccess) e = cudaMemcpy(dx, X, 4ull * n * d.D, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const unsigned tiles = (unsigned)((n + kTile - 1) / kTile);
        mlp_forward_kernel<<<tiles, d.H, fwd_smem(d)>>>(d, M->P, dx, n, dy);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(Y, dy, 4ull * n * d.O, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    return e == cudaSuccess ? ES_OK : mlp_fail(ES_ERR_CUDA, cudaGetErrorString(e));
}

// Full-batch loss (mean squared error) and its gradient with respect to every parameter.
int es_mlp_loss_grad(es_mlp* M, const float* X, const float* T, uint64_t n, float* loss, float* grad) {
    if (!M || !X || !T || n == 0 || !loss) return mlp_fail(ES_ERR_ARG, "null argument or empty set");
    const Dims d = M->d;
    const int np = d.n();
    const unsigned tiles = (unsigned)((n + kTile - 1) / kTile);
    float *dx = nullptr, *dt = nullptr, *G = nullptr, *L = nullptr;
    cudaError_t e = cudaMalloc(&dx, 4ull * n * d.D);
    if (e == cudaSuccess) e = cudaMalloc(&dt, 4ull * n * d.O);
    if (e == cudaSuccess) e = cudaMalloc(&G, 4ull * tiles * np);
    if (e == cudaSuccess) e = cudaMalloc(&L, 4ull * tiles);
    if (e == cudaSuccess) e = cudaMemcpy(dx, X, 4ull * n * d.D, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dt, T, 4ull * n * d.O, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const float scale = 1.f / (float)(n * d.O);
        mlp_grad_kernel<<<tiles, d.H, grad_smem(d)>>>(d, M->P, dx, dt, nullptr, n, scale, G, L);
        mlp_reduce_kernel<<<(np + 255) / 256, 256>>>(G, (int)tiles, np, M->g, L, M->loss);
        e = cudaGetLastError();
    }
    float l = 0.f;
    if (e == cudaSuccess) e = cudaMemcpy(&l, M->loss, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && grad) e = cudaMemcpy(grad, M->g, 4ull * np, cudaMemcpyDeviceToHost);
    *loss = l / (float)(n * d.O);
    cudaFree(dx); cudaFree(dt); cudaFree(G); cudaFree(L);
    return e == cudaSuccess ? ES_OK : mlp_fail(ES_ERR_CUDA, cudaGetErrorString(e));
}

// Minibatch Adam on (X, T): `epochs` passes over a seeded permutation, `batch` samples a step.
int es_mlp_train(es_mlp* M, const float* X, const float* T, uint64_t n, uint32_t epochs, uint32_t batch,
                 float lr, uint64_t seed, float* final_loss) {
    if (!M || !X || !T || n == 0 || batch == 0) return mlp_fail(ES_ERR_ARG, "null argument or empty set");
    const Dims d = M->d;
    const int np = d.n();
    const unsigned max_tiles = (unsigned)((batch + kTile - 1) / kTile);
    float *dx = nullptr, *dt = nullptr, *G = nullptr, *L = nullptr;
    uint32_t* didx = nullptr;
    cudaError_t e = cudaMalloc(&dx, 4ull * n * d.D);
    if (e == cudaSuccess) e = cudaMalloc(&dt, 4ull * n * d.O);
    if (e == cudaSuccess) e = cudaMalloc(&G, 4ull * max_tiles * np);
    if (e == cudaSuccess) e = cudaMalloc(&L, 4ull * max_tiles);
    if (e == cudaSuccess) e = cudaMalloc(&didx, 4ull * n);
    if (e == cudaSuccess) e = cudaMemcpy(dx, X, 4ull * n * d.D, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dt, T, 4ull * n * d.O, cudaMemcpyHostToDevice);
    std::vector<uint32_t> perm(n);
    for (uint64_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
    uint64_t s = seed;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (uint32_t ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
        for (uint64_t i = n - 1; i > 0; --i) {   // Fisher-Yates with a seeded generator
            const uint64_t j = splitmix(s) % (i + 1);
            std::swap(perm[i], perm[j]);
        }
        e = cudaMemcpy(didx, perm.data(), 4ull * n, cudaMemcpyHostToDevice);
        for (uint64_t b0 = 0; b0 < n && e == cudaSuccess; b0 += batch) {
            const uint64_t nb = (n - b0) < batch ? (n - b0) : batch;
            const unsigned tiles = (unsigned)((nb + kTile - 1) / kTile);
            const float scale = 1.f / (float)(nb * d.O);
            mlp_grad_kernel<<<tiles, d.H, grad_smem(d)>>>(d, M->P, dx, dt, didx + b0, nb, scale, G, L);
            mlp_reduce_kernel<<<(np + 255) / 256, 256>>>(G, (int)tiles, np, M->g, L, M->loss);
            M->steps += 1;
            const float c1 = 1.f - std::pow(b1, (float)M->steps), c2 = 1.f - std::pow(b2, (float)M->steps);
            mlp_adam_kernel<<<(np + 255) / 256, 256>>>(M->P, M->g, M->m, M->v, np, lr, b1, b2, eps, c1, c2);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (final_loss && e == cudaSuccess) {
        cudaFree(G);
        G = nullptr;
        float l = 0.f;
        int r = es_mlp_loss_grad(M, X, T, n, &l, nullptr);
        if (r) { cudaFree(dx); cudaFree(dt); cudaFree(L); cudaFree(didx); return r; }
        *final_loss = l;
    }
    cudaFree(dx); cudaFree(dt); cudaFree(G); cudaFree(L); cudaFree(didx);
    return e == cudaSuccess ? ES_OK : mlp_fail(ES_ERR_CUDA, cudaGetErrorString(e));
}

}  // extern "C"
