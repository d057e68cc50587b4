// galp_mlp.cu -- the dispatcher's MLP as a trainable object behind the C ABI
// (include/galp_tools.h): forward, loss gradient and AdamW training, all on the GPU with
// the FP32 kernels of mlp_kernels.cuh.  Three layers: nin -> nhid -> nhid -> nout, ReLU
// after the first two, masked mean squared error on the outputs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/galp.h"
#include "../../include/galp_tools.h"
#include "mlp_kernels.cuh"

using namespace galp;

namespace {

int mlp_status(cudaError_t e)
{
    if (e == cudaSuccess) return GALP_OK;
    if (e == cudaErrorMemoryAllocation) return GALP_ENOMEM;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GALP_ENODEV;
    return GALP_ECUDA;
}

#define MLP_CUDA(call)                                  \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return mlp_status(e_);   \
    } while (0)

struct Buf {
    float *p = nullptr;
    int64_t n = 0;
    ~Buf()
    {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(int64_t count)
    {
        if (count <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, sizeof(float) * (size_t)std::max<int64_t>(count, 1));
        if (e == cudaSuccess) n = count;
        return e;
    }
};

unsigned grid_for(int64_t work, int block = 256)
{
    return (unsigned)std::min<int64_t>((work + block - 1) / block, 65535);
}

}  // namespace

struct galp_mlp {
    int nin = 0, nhid = 0, nout = 0;
    int64_t np = 0;
    Buf w, g, m1, m2;                      // parameters, gradient, Adam moments
    Buf x, t, mask, h1, h2, y, d3, d2, d1, loss;
    int64_t step = 0;
    cudaStream_t st = nullptr;

    // parameter blocks
    float *W1(float *b) const { return b; }
    float *B1(float *b) const { return b + (int64_t)nin * nhid; }
    float *W2(float *b) const { return B1(b) + nhid; }
    float *B2(float *b) const { return W2(b) + (int64_t)nhid * nhid; }
    float *W3(float *b) const { return B2(b) + nhid; }
    float *B3(float *b) const { return W3(b) + (int64_t)nhid * nout; }

    int upload_batch(const float *hx, const float *ht, const float *hm, int B)
    {
        MLP_CUDA(x.ensure((int64_t)B * nin));
        MLP_CUDA(cudaMemcpyAsync(x.p, hx, sizeof(float) * B * nin, cudaMemcpyHostToDevice, st));
        if (ht) {
            MLP_CUDA(t.ensure((int64_t)B * nout));
            MLP_CUDA(mask.ensure((int64_t)B * nout));
            MLP_CUDA(cudaMemcpyAsync(t.p, ht, sizeof(float) * B * nout, cudaMemcpyHostToDevice, st));
            if (hm) {
                MLP_CUDA(cudaMemcpyAsync(mask.p, hm, sizeof(float) * B * nout, cudaMemcpyHostToDevice, st));
            } else {
                std::vector<float> ones((size_t)B * nout, 1.f);
                MLP_CUDA(cudaMemcpyAsync(mask.p, ones.data(), sizeof(float) * B * nout, cudaMemcpyHostToDevice, st));
                MLP_CUDA(cudaStreamSynchronize(st));
            }
        }
        MLP_CUDA(h1.ensure((int64_t)B * nhid));
        MLP_CUDA(h2.ensure((int64_t)B * nhid));
        MLP_CUDA(y.ensure((int64_t)B * nout));
        MLP_CUDA(d3.ensure((int64_t)B * nout));
        MLP_CUDA(d2.ensure((int64_t)B * nhid));
        MLP_CUDA(d1.ensure((int64_t)B * nhid));
        MLP_CUDA(loss.ensure(1));
        return GALP_OK;
    }

    void forward(int B)
    {
        mlp_linear_fwd<<<grid_for((int64_t)B * nhid), 256, 0, st>>>(x.p, W1(w.p), B1(w.p), h1.p, B, nin, nhid, 1);
        mlp_linear_fwd<<<grid_for((int64_t)B * nhid), 256, 0, st>>>(h1.p, W2(w.p), B2(w.p), h2.p, B, nhid, nhid, 1);
        mlp_linear_fwd<<<grid_for((int64_t)B * nout), 256, 0, st>>>(h2.p, W3(w.p), B3(w.p), y.p, B, nhid, nout, 0);
    }

    // gradient of the masked MSE into g; loss into loss.p[0]
    void backward(int B, float inv_count)
    {
        cudaMemsetAsync(loss.p, 0, sizeof(float), st);
        const int64_t tot = (int64_t)B * nout;
        mlp_mse_grad<<<std::min<unsigned>(grid_for(tot), 1024), 256, 0, st>>>(y.p, t.p, mask.p, d3.p, tot, inv_count,
                                                                              loss.p);
        mlp_linear_wgrad<<<grid_for((int64_t)(nhid + 1) * nout), 256, 0, st>>>(h2.p, d3.p, W3(g.p), B3(g.p), B, nhid,
                                                                                nout);
        mlp_linear_xgrad<<<grid_for((int64_t)B * nhid), 256, 0, st>>>(d3.p, W3(w.p), d2.p, B, nhid, nout);
        mlp_relu_bwd<<<std::min<unsigned>(grid_for((int64_t)B * nhid), 1024), 256, 0, st>>>(d2.p, h2.p,
                                                                                             (int64_t)B * nhid);
        mlp_linear_wgrad<<<grid_for((int64_t)(nhid + 1) * nhid), 256, 0, st>>>(h1.p, d2.p, W2(g.p), B2(g.p), B, nhid,
                                                                                nhid);
        mlp_linear_xgrad<<<grid_for((int64_t)B * nhid), 256, 0, st>>>(d2.p, W2(w.p), d1.p, B, nhid, nhid);
        mlp_relu_bwd<<<std::min<unsigned>(grid_for((int64_t)B * nhid), 1024), 256, 0, st>>>(d1.p, h1.p,
                                                                                             (int64_t)B * nhid);
        mlp_linear_wgrad<<<grid_for((int64_t)(nin + 1) * nhid), 256, 0, st>>>(x.p, d1.p, W1(g.p), B1(g.p), B, nin,
                                                                               nhid);
    }
};

namespace {

float mask_count(const float *hm, int64_t total)
{
    if (!hm) return (float)total;
    double c = 0;
    for (int64_t i = 0; i < total; ++i) c += hm[i];
    return (float)std::max(c, 1.0);
}

}  // namespace

extern "C" {

int64_t galp_mlp_size(int32_t nin, int32_t nhid, int32_t nout)
{
    if (nin <= 0 || nhid <= 0 || nout <= 0) return 0;
    return mlp_param_count(nin, nhid, nout);
}

int galp_mlp_create(int32_t nin, int32_t nhid, int32_t nout, uint64_t seed, galp_mlp **out)
{
    if (!out || nin <= 0 || nhid <= 0 || nout <= 0 || nin > 4096 || nhid > 4096 || nout > 4096) return GALP_EINVAL;
    *out = nullptr;
    galp_mlp *M = new (std::nothrow) galp_mlp();
    if (!M) return GALP_ENOMEM;
    M->nin = nin;
    M->nhid = nhid;
    M->nout = nout;
    M->np = mlp_param_count(nin, nhid, nout);
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&M->st, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = M->w.ensure(M->np)) != cudaSuccess || (e = M->g.ensure(M->np)) != cudaSuccess ||
        (e = M->m1.ensure(M->np)) != cudaSuccess || (e = M->m2.ensure(M->np)) != cudaSuccess) {
        const int rc = mlp_status(e);
        galp_mlp_destroy(M);
        return rc;
    }
    // He-uniform initial weights from a splitmix64 stream, zero biases
    std::vector<float> h((size_t)M->np, 0.f);
    uint64_t s = seed;
    auto uni = [&s]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) / 9007199254740992.0;  // [0, 1)
    };
    auto fill = [&](float *p, int fan_in, int64_t cnt) {
        const double a = std::sqrt(6.0 / fan_in);
        for (int64_t i = 0; i < cnt; ++i) p[i] = (float)((2.0 * uni() - 1.0) * a);
    };
    fill(M->W1(h.data()), nin, (int64_t)nin * nhid);
    fill(M->W2(h.data()), nhid, (int64_t)nhid * nhid);
    fill(M->W3(h.data()), nhid, (int64_t)nhid * nout);
    int rc = galp_mlp_set_weights(M, h.data(), M->np);
    if (rc) {
        galp_mlp_destroy(M);
        return rc;
    }
    *out = M;
    return GALP_OK;
}

int galp_mlp_set_weights(galp_mlp *M, const float *w, int64_t count)
{
    if (!M || !w || count != M->np) return GALP_EINVAL;
    MLP_CUDA(cudaMemcpyAsync(M->w.p, w, sizeof(float) * count, cudaMemcpyHostToDevice, M->st));
    MLP_CUDA(cudaMemsetAsync(M->m1.p, 0, sizeof(float) * count, M->st));
    MLP_CUDA(cudaMemsetAsync(M->m2.p, 0, sizeof(float) * count, M->st));
    MLP_CUDA(cudaStreamSynchronize(M->st));
    M->step = 0;
    return GALP_OK;
}

int galp_mlp_get_weights(galp_mlp *M, float *w, int64_t count)
{
    if (!M || !w || count != M->np) return GALP_EINVAL;
    MLP_CUDA(cudaMemcpyAsync(w, M->w.p, sizeof(float) * count, cudaMemcpyDeviceToHost, M->st));
    MLP_CUDA(cudaStreamSynchronize(M->st));
    return GALP_OK;
}

int galp_mlp_forward(galp_mlp *M, const float *x, int32_t batch, float *y)
{
    if (!M || !x || !y || batch <= 0) return GALP_EINVAL;
    int rc = M->upload_batch(x, nullptr, nullptr, batch);
    if (rc) return rc;
    M->forward(batch);
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpyAsync(y, M->y.p, sizeof(float) * batch * M->nout, cudaMemcpyDeviceToHost, M->st));
    MLP_CUDA(cudaStreamSynchronize(M->st));
    return GALP_OK;
}

int galp_mlp_loss_grad(galp_mlp *M, const float *x, const float *t, const float *mask, int32_t batch, float *loss,
                       float *grad)
{
    if (!M || !x || !t || !loss || !grad || batch <= 0) return GALP_EINVAL;
    int rc = M->upload_batch(x, t, mask, batch);
    if (rc) return rc;
    M->forward(batch);
    M->backward(batch, 1.f / mask_count(mask, (int64_t)batch * M->nout));
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpyAsync(loss, M->loss.p, sizeof(float), cudaMemcpyDeviceToHost, M->st));
    MLP_CUDA(cudaMemcpyAsync(grad, M->g.p, sizeof(float) * M->np, cudaMemcpyDeviceToHost, M->st));
    MLP_CUDA(cudaStreamSynchronize(M->st));
    return GALP_OK;
}

int galp_mlp_train(galp_mlp *M, const float *x, const float *t, const float *mask, int32_t batch, int32_t steps,
                   float lr, float weight_decay, float *loss_curve)
{
    if (!M || !x || !t || batch <= 0 || steps < 0 || !(lr > 0.f)) return GALP_EINVAL;
    int rc = M->upload_batch(x, t, mask, batch);
    if (rc) return rc;
    const float inv = 1.f / mask_count(mask, (int64_t)batch * M->nout);
    const float b1 = 0.9f, b2 = 0.999f;
    for (int s = 0; s < steps; ++s) {
        M->forward(batch);
        M->backward(batch, inv);
        ++M->step;
        const float c1 = 1.f - std::pow(b1, (float)M->step), c2 = 1.f - std::pow(b2, (float)M->step);
        mlp_adam<<<grid_for(M->np), 256, 0, M->st>>>(M->w.p, M->g.p, M->m1.p, M->m2.p, M->np, lr, b1, b2, 1e-8f,
                                                     weight_decay, c1, c2);
        if (loss_curve) MLP_CUDA(cudaMemcpyAsync(&loss_curve[s], M->loss.p, sizeof(float), cudaMemcpyDeviceToHost, M->st));
    }
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaStreamSynchronize(M->st));
    return GALP_OK;
}

void galp_mlp_destroy(galp_mlp *M)
{
    if (!M) return;
    if (M->st) cudaStreamSynchronize(M->st);
    if (M->st) cudaStreamDestroy(M->st);
    delete M;
}

}  // extern "C"
