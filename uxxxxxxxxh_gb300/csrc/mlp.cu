// Cost-model network: a small fully connected MLP (in -> H -> ... -> H -> 1,
// ReLU between layers) trained and evaluated on the GPU by the kernels in
// this file.  It predicts a launch configuration's time per point from the
// program's and the launch's features (uxxxxxxxxh_gb300/costmodel.py).
//
// Layout: one flat float buffer of parameters, layer by layer
// [W (out x in, row-major), b (out)], on the device.  Activations of the
// last forward pass are kept for the backward pass.  Every reduction is a
// plain loop in one thread (no atomics), so forward, loss and gradients are
// deterministic and can be compared against a CPU implementation exactly up
// to float rounding.  Training is Adam on the mean squared error, minibatches
// drawn from a fixed device-resident data set by a seeded permutation.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>

#include "uhs_kernels.h"

namespace uhs {
int set_error(int code, const char *fmt, ...);
}

struct uhs_mlp {
    int in_dim = 0, hidden = 0, layers = 0;  // layers = number of hidden layers
    std::vector<int> dims;                   // in, H, ..., H, 1
    std::vector<int64_t> off;                // parameter offset of each layer's W
    int64_t nparam = 0;
    float *w = nullptr;       // parameters
    float *g = nullptr;       // gradients
    float *m = nullptr;       // Adam first moment
    float *v = nullptr;       // Adam second moment
    int64_t step = 0;
    // work buffers sized for `cap` rows
    int64_t cap = 0;
    std::vector<float *> act;  // act[l]: input of layer l (act[0] = x); act[L]: output
    std::vector<float *> dact;
    float *y = nullptr;
    float *loss = nullptr;
};

namespace uhs {
namespace {

constexpr int kT = 256;

// Y[n][o] = act(b[o] + sum_i X[n][i] W[o][i])
__global__ void k_linear_fwd(const float *__restrict__ X, const float *__restrict__ W, const float *__restrict__ b,
                             float *__restrict__ Y, int n, int din, int dout, int relu) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(n) * dout) return;
    const int r = static_cast<int>(t / dout), o = static_cast<int>(t % dout);
    const float *x = X + static_cast<int64_t>(r) * din;
    const float *w = W + static_cast<int64_t>(o) * din;
    float s = b[o];
    for (int i = 0; i < din; ++i) s = fmaf(x[i], w[i], s);
    Y[t] = relu && s < 0.0f ? 0.0f : s;
}

// dY of the loss L = mean((p - y)^2): 2 (p - y) / n, and the loss itself.
__global__ void k_mse_grad(const float *__restrict__ p, const float *__restrict__ y, float *__restrict__ dp, int n,
                           float *__restrict__ loss) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dp[t] = 2.0f * (p[t] - y[t]) / static_cast<float>(n);
    if (t == 0) {
        float s = 0.0f;
        for (int i = 0; i < n; ++i) {
            const float d = p[i] - y[i];
            s = fmaf(d, d, s);
        }
        *loss = s / static_cast<float>(n);
    }
}

// dZ = dY masked by the ReLU of the layer output Y (in place).
__global__ void k_relu_bwd(float *__restrict__ dY, const float *__restrict__ Y, int64_t count) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t < count && Y[t] <= 0.0f) dY[t] = 0.0f;
}

// dW[o][i] = sum_n dZ[n][o] X[n][i];  db[o] = sum_n dZ[n][o]
__global__ void k_linear_bwd_w(const float *__restrict__ dZ, const float *__restrict__ X, float *__restrict__ dW,
                               float *__restrict__ db, int n, int din, int dout) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < dout * din) {
        const int o = t / din, i = t % din;
        float s = 0.0f;
        for (int r = 0; r < n; ++r) s = fmaf(dZ[static_cast<int64_t>(r) * dout + o], X[static_cast<int64_t>(r) * din + i], s);
        dW[t] = s;
    } else if (t < dout * din + dout) {
        const int o = t - dout * din;
        float s = 0.0f;
        for (int r = 0; r < n; ++r) s += dZ[static_cast<int64_t>(r) * dout + o];
        db[o] = s;
    }
}

// dX[n][i] = sum_o dZ[n][o] W[o][i]
__global__ void k_linear_bwd_x(const float *__restrict__ dZ, const float *__restrict__ W, float *__restrict__ dX,
                               int n, int din, int dout) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(n) * din) return;
    const int r = static_cast<int>(t / din), i = static_cast<int>(t % din);
    float s = 0.0f;
    for (int o = 0; o < dout; ++o) s = fmaf(dZ[static_cast<int64_t>(r) * dout + o], W[static_cast<int64_t>(o) * din + i], s);
    dX[t] = s;
}

__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m, float *__restrict__ v,
                       int64_t n, float lr, float b1, float b2, float c1, float c2, float eps) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= n) return;
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.0f - b1) * gt;
    const float vt = b2 * v[t] + (1.0f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    w[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
}

// Gather rows idx[0..n) of X (din wide) and y into contiguous buffers.
__global__ void k_gather(const float *__restrict__ X, const float *__restrict__ y, const int *__restrict__ idx,
                         float *__restrict__ Xo, float *__restrict__ yo, int n, int din) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= static_cast<int64_t>(n) * din) return;
    const int r = static_cast<int>(t / din), i = static_cast<int>(t % din);
    const int s = idx[r];
    Xo[t] = X[static_cast<int64_t>(s) * din + i];
    if (i == 0) yo[r] = y[s];
}

unsigned blocks(int64_t n) { return static_cast<unsigned>((n + kT - 1) / kT); }

cudaError_t reserve(uhs_mlp *m, int64_t rows) {
    if (rows <= m->cap) return cudaSuccess;
    for (auto *p : m->act) cudaFree(p);
    for (auto *p : m->dact) cudaFree(p);
    cudaFree(m->y);
    m->act.assign(m->dims.size(), nullptr);
    m->dact.assign(m->dims.size(), nullptr);
    for (size_t l = 0; l < m->dims.size(); ++l) {
        if (dev_alloc((void **)&m->act[l], sizeof(float) * rows * m->dims[l]) != cudaSuccess) return cudaErrorMemoryAllocation;
        if (dev_alloc((void **)&m->dact[l], sizeof(float) * rows * m->dims[l]) != cudaSuccess) return cudaErrorMemoryAllocation;
    }
    if (dev_alloc((void **)&m->y, sizeof(float) * rows) != cudaSuccess) return cudaErrorMemoryAllocation;
    m->cap = rows;
    return cudaSuccess;
}

// Forward over act[0] (n rows); output in act[L].
void forward(uhs_mlp *m, int n) {
    const int L = static_cast<int>(m->dims.size()) - 1;
    for (int l = 0; l < L; ++l) {
        const int din = m->dims[l], dout = m->dims[l + 1];
        const float *W = m->w + m->off[l];
        k_linear_fwd<<<blocks(static_cast<int64_t>(n) * dout), kT>>>(m->act[l], W, W + static_cast<int64_t>(dout) * din,
                                                                      m->act[l + 1], n, din, dout, l + 1 < L);
    }
    count_launch(L);
}

// Loss and gradients (into m->g) for the rows in act[0] with targets m->y.
void backward(uhs_mlp *m, int n) {
    const int L = static_cast<int>(m->dims.size()) - 1;
    k_mse_grad<<<blocks(n), kT>>>(m->act[L], m->y, m->dact[L], n, m->loss);
    for (int l = L - 1; l >= 0; --l) {
        const int din = m->dims[l], dout = m->dims[l + 1];
        if (l + 1 < L) k_relu_bwd<<<blocks(static_cast<int64_t>(n) * dout), kT>>>(m->dact[l + 1], m->act[l + 1],
                                                                                  static_cast<int64_t>(n) * dout);
        float *dW = m->g + m->off[l];
        k_linear_bwd_w<<<blocks(static_cast<int64_t>(dout) * din + dout), kT>>>(
            m->dact[l + 1], m->act[l], dW, dW + static_cast<int64_t>(dout) * din, n, din, dout);
        if (l > 0)
            k_linear_bwd_x<<<blocks(static_cast<int64_t>(n) * din), kT>>>(m->dact[l + 1], m->w + m->off[l], m->dact[l],
                                                                          n, din, dout);
    }
    count_launch(3 * L + 1);
}

}  // namespace
}  // namespace uhs

using uhs::dev_alloc;
using uhs::set_error;

extern "C" {

int uhs_mlp_create(int32_t in_dim, int32_t hidden, int32_t layers, uint64_t seed, uhs_mlp **out) {
    if (!out || in_dim < 1 || hidden < 1 || layers < 1 || in_dim > 4096 || hidden > 4096 || layers > 16)
        return set_error(UHS_EINVAL, "bad MLP shape (in %d, hidden %d, layers %d)", in_dim, hidden, layers);
    auto *m = new uhs_mlp();
    m->in_dim = in_dim;
    m->hidden = hidden;
    m->layers = layers;
    m->dims.push_back(in_dim);
    for (int i = 0; i < layers; ++i) m->dims.push_back(hidden);
    m->dims.push_back(1);
    for (size_t l = 0; l + 1 < m->dims.size(); ++l) {
        m->off.push_back(m->nparam);
        m->nparam += static_cast<int64_t>(m->dims[l + 1]) * (m->dims[l] + 1);
    }
    // He-uniform initial weights, zero biases (host RNG, seeded)
    std::vector<float> h(static_cast<size_t>(m->nparam), 0.0f);
    std::mt19937_64 rng(seed);
    for (size_t l = 0; l + 1 < m->dims.size(); ++l) {
        const int din = m->dims[l], dout = m->dims[l + 1];
        const float lim = std::sqrt(6.0f / static_cast<float>(din));
        std::uniform_real_distribution<float> U(-lim, lim);
        for (int64_t i = 0; i < static_cast<int64_t>(din) * dout; ++i) h[m->off[l] + i] = U(rng);
    }
    const size_t bytes = sizeof(float) * static_cast<size_t>(m->nparam);
    if (dev_alloc((void **)&m->w, bytes) || dev_alloc((void **)&m->g, bytes) || dev_alloc((void **)&m->m, bytes) ||
        dev_alloc((void **)&m->v, bytes) || dev_alloc((void **)&m->loss, sizeof(float))) {
        delete m;
        return set_error(UHS_ENOMEM, "MLP allocation failed");
    }
    cudaMemcpy(m->w, h.data(), bytes, cudaMemcpyHostToDevice);
    cudaMemset(m->g, 0, bytes);
    cudaMemset(m->m, 0, bytes);
    cudaMemset(m->v, 0, bytes);
    *out = m;
    return UHS_OK;
}

void uhs_mlp_destroy(uhs_mlp *m) {
    if (!m) return;
    for (auto *p : m->act) cudaFree(p);
    for (auto *p : m->dact) cudaFree(p);
    cudaFree(m->y);
    cudaFree(m->w);
    cudaFree(m->g);
    cudaFree(m->m);
    cudaFree(m->v);
    cudaFree(m->loss);
    delete m;
}

int64_t uhs_mlp_num_params(const uhs_mlp *m) { return m ? m->nparam : 0; }

int uhs_mlp_get_params(const uhs_mlp *m, float *out) {
    if (!m || !out) return set_error(UHS_EINVAL, "NULL argument");
    if (cudaMemcpy(out, m->w, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_error(UHS_ECUDA, "parameter read failed");
    return UHS_OK;
}

int uhs_mlp_set_params(uhs_mlp *m, const float *in) {
    if (!m || !in) return set_error(UHS_EINVAL, "NULL argument");
    if (cudaMemcpy(m->w, in, sizeof(float) * m->nparam, cudaMemcpyHostToDevice) != cudaSuccess)
        return set_error(UHS_ECUDA, "parameter write failed");
    m->step = 0;
    cudaMemset(m->m, 0, sizeof(float) * m->nparam);
    cudaMemset(m->v, 0, sizeof(float) * m->nparam);
    return UHS_OK;
}

int uhs_mlp_forward(uhs_mlp *m, const float *x, int32_t n, float *y) {
    if (!m || !x || !y || n < 0) return set_error(UHS_EINVAL, "NULL argument or negative n");
    if (n == 0) return UHS_OK;
    if (uhs::reserve(m, n) != cudaSuccess) return set_error(UHS_ENOMEM, "MLP work buffers");
    cudaMemcpy(m->act[0], x, sizeof(float) * n * m->in_dim, cudaMemcpyHostToDevice);
    uhs::forward(m, n);
    const cudaError_t e = cudaMemcpy(y, m->act.back(), sizeof(float) * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return set_error(UHS_ECUDA, "MLP forward: %s", cudaGetErrorString(e));
    return UHS_OK;
}

int uhs_mlp_loss_grad(uhs_mlp *m, const float *x, const float *y, int32_t n, float *loss, float *grad) {
    if (!m || !x || !y || n < 1) return set_error(UHS_EINVAL, "NULL argument or empty batch");
    if (uhs::reserve(m, n) != cudaSuccess) return set_error(UHS_ENOMEM, "MLP work buffers");
    cudaMemcpy(m->act[0], x, sizeof(float) * n * m->in_dim, cudaMemcpyHostToDevice);
    cudaMemcpy(m->y, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    uhs::forward(m, n);
    uhs::backward(m, n);
    cudaError_t e = cudaSuccess;
    if (loss) e = cudaMemcpy(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && grad) e = cudaMemcpy(grad, m->g, sizeof(float) * m->nparam, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return set_error(UHS_ECUDA, "MLP gradient: %s", cudaGetErrorString(e));
    return UHS_OK;
}

int uhs_mlp_train(uhs_mlp *m, const float *x, const float *y, int32_t n, int32_t epochs, int32_t batch, float lr,
                  uint64_t seed, float *final_loss) {
    if (!m || !x || !y || n < 1 || epochs < 0 || batch < 1) return set_error(UHS_EINVAL, "bad training arguments");
    batch = std::min(batch, n);
    float *dx = nullptr, *dy = nullptr;
    int *didx = nullptr;
    if (dev_alloc((void **)&dx, sizeof(float) * n * m->in_dim) || dev_alloc((void **)&dy, sizeof(float) * n) ||
        dev_alloc((void **)&didx, sizeof(int) * n)) {
        cudaFree(dx);
        cudaFree(dy);
        return set_error(UHS_ENOMEM, "training set upload");
    }
    cudaMemcpy(dx, x, sizeof(float) * n * m->in_dim, cudaMemcpyHostToDevice);
    cudaMemcpy(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    if (uhs::reserve(m, batch) != cudaSuccess) {
        cudaFree(dx);
        cudaFree(dy);
        cudaFree(didx);
        return set_error(UHS_ENOMEM, "MLP work buffers");
    }
    std::vector<int> perm(static_cast<size_t>(n));
    std::mt19937_64 rng(seed);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int i = 0; i < n; ++i) perm[i] = i;
        std::shuffle(perm.begin(), perm.end(), rng);
        cudaMemcpy(didx, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
        for (int s = 0; s + batch <= n; s += batch) {
            uhs::k_gather<<<uhs::blocks(static_cast<int64_t>(batch) * m->in_dim), uhs::kT>>>(
                dx, dy, didx + s, m->act[0], m->y, batch, m->in_dim);
            uhs::forward(m, batch);
            uhs::backward(m, batch);
            ++m->step;
            const float c1 = 1.0f - std::pow(b1, static_cast<float>(m->step));
            const float c2 = 1.0f - std::pow(b2, static_cast<float>(m->step));
            uhs::k_adam<<<uhs::blocks(m->nparam), uhs::kT>>>(m->w, m->g, m->m, m->v, m->nparam, lr, b1, b2, c1, c2,
                                                            eps);
            uhs::count_launch(2);
        }
    }
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess && final_loss) e = cudaMemcpy(final_loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(didx);
    if (e != cudaSuccess) return set_error(UHS_ECUDA, "MLP training: %s", cudaGetErrorString(e));
    return UHS_OK;
}

}  // extern "C"
