// host_selector.cpp -- the learned TENO stencil selector behind the C ABI:
// dataset harvest from a solver context, minibatch training on the GPU,
// tensor-core inference and its attachment to an FP32-form context.
//
// The selector has no counterpart in the reference.  Its labels are the
// decisions of the corrected TENO form (face_reconstruction.cpp:939-981 with
// the cut-off weights fixed) computed by the FP64 kernels on the solver's
// own states.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <random>
#include <vector>

#include "host_ctx.h"
#include "selector_params.h"
#include "selector_launch.h"

using namespace mgpu;

struct mgpu_selector {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<float> params;  // host copy, authoritative between calls
    DevArray<float> d_params, d_grad, d_m, d_v;
    uint32_t adam_t = 0;
    DevArray<uint8_t> d_wimg;
    bool wimg_dirty = true;
    // dataset
    DevArray<float> X;
    DevArray<uint8_t> Y;
    size_t n = 0, cap = 0;
    // batch work
    size_t wb = 0;
    DevArray<float> Xb, Z1, A1, Z2, A2, Z3, dZ3, dA, dZ, work, part;
    DevArray<uint8_t> Yb;
    DevArray<uint32_t> perm;
    DevArray<unsigned> err;

    ~mgpu_selector() {
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace mgpu {
namespace {

uint16_t bf16_rn(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    b += 0x7FFFu + ((b >> 16) & 1u);
    return (uint16_t)(b >> 16);
}

// BF16 weight image in the no-swizzle K-major core-matrix layout the
// inference kernel hands to tcgen05.mma (B operand = W^T: row n, column k),
// followed by the FP32 biases.
std::vector<uint8_t> weight_image(const std::vector<float>& p) {
    std::vector<uint8_t> img(sel::WEIGHT_IMAGE_BYTES, 0);
    auto put = [&](size_t base, const float* W, int K, int N) {
        for (int nn = 0; nn < N; ++nn)
            for (int k = 0; k < K; ++k) {
                const size_t off = base + (size_t)(((nn >> 3) * (K >> 3) + (k >> 3)) * 128 + (nn & 7) * 16 + (k & 7) * 2);
                const uint16_t h = bf16_rn(W[(size_t)k * N + nn]);
                std::memcpy(&img[off], &h, 2);
            }
    };
    put(0, p.data() + sel::OFF_W1, sel::IN, sel::HID);
    put((size_t)sel::HID * sel::IN * 2, p.data() + sel::OFF_W2, sel::HID, sel::HID);
    put((size_t)sel::HID * sel::IN * 2 + (size_t)sel::HID * sel::HID * 2, p.data() + sel::OFF_W3, sel::HID, sel::OUT);
    size_t off = (size_t)sel::HID * sel::IN * 2 + (size_t)sel::HID * sel::HID * 2 + (size_t)sel::OUT * sel::HID * 2;
    std::memcpy(&img[off], p.data() + sel::OFF_B1, sel::HID * 4);
    off += sel::HID * 4;
    std::memcpy(&img[off], p.data() + sel::OFF_B2, sel::HID * 4);
    off += sel::HID * 4;
    std::memcpy(&img[off], p.data() + sel::OFF_B3, sel::OUT * 4);
    return img;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        ck(cudaSetDevice(dev), "cudaSetDevice");
    }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

void upload_params(mgpu_selector* s) {
    ck(cudaMemcpyAsync(s->d_params.p, s->params.data(), s->params.size() * 4, cudaMemcpyHostToDevice, s->stream),
       "H2D params");
    s->wimg_dirty = true;
}

void download_params(mgpu_selector* s) {
    ck(cudaMemcpyAsync(s->params.data(), s->d_params.p, s->params.size() * 4, cudaMemcpyDeviceToHost, s->stream),
       "D2H params");
    ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
}

void refresh_image(mgpu_selector* s) {
    if (!s->wimg_dirty) return;
    const std::vector<uint8_t> img = weight_image(s->params);
    ck(cudaMemcpyAsync(s->d_wimg.p, img.data(), img.size(), cudaMemcpyHostToDevice, s->stream), "H2D image");
    ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    s->wimg_dirty = false;
}

void ensure_batch(mgpu_selector* s, size_t rows) {
    if (rows <= s->wb) return;
    s->Xb.alloc(rows * sel::IN);
    s->Yb.alloc(rows * sel::NV);
    s->Z1.alloc(rows * sel::HID);
    s->A1.alloc(rows * sel::HID);
    s->Z2.alloc(rows * sel::HID);
    s->A2.alloc(rows * sel::HID);
    s->Z3.alloc(rows * sel::OUT);
    s->dZ3.alloc(rows * sel::OUT);
    s->dA.alloc(rows * sel::HID);
    s->dZ.alloc(rows * sel::HID);
    s->wb = rows;
}

constexpr int SPLITS = 16;

// Forward and backward of one batch already in Xb/Yb; gradient into d_grad,
// per-block loss sums into part (xent_blocks(rows) floats).
void forward_backward(mgpu_selector* s, int rows, float* part) {
    using namespace sel;
    cudaStream_t st = s->stream;
    float* P = s->d_params.p;
    float* G = s->d_grad.p;
    // forward
    ck(launch_sgemm(false, false, rows, HID, IN, s->Xb.p, IN, P + OFF_W1, HID, s->Z1.p, HID, false, 1, nullptr, st),
       "sgemm");
    ck(launch_bias_act(rows, HID, s->Z1.p, P + OFF_B1, s->A1.p, true, st), "bias_act");
    ck(launch_sgemm(false, false, rows, HID, HID, s->A1.p, HID, P + OFF_W2, HID, s->Z2.p, HID, false, 1, nullptr, st),
       "sgemm");
    ck(launch_bias_act(rows, HID, s->Z2.p, P + OFF_B2, s->A2.p, true, st), "bias_act");
    ck(launch_sgemm(false, false, rows, OUT, HID, s->A2.p, HID, P + OFF_W3, OUT, s->Z3.p, OUT, false, 1, nullptr, st),
       "sgemm");
    ck(launch_bias_act(rows, OUT, s->Z3.p, P + OFF_B3, nullptr, false, st), "bias");
    ck(launch_xent(rows, s->Z3.p, s->Yb.p, 1.0f / (float)(rows * NV), s->dZ3.p, part, st), "xent");
    // backward
    ck(launch_sgemm(true, false, HID, OUT, rows, s->A2.p, HID, s->dZ3.p, OUT, G + OFF_W3, OUT, false, SPLITS,
                    s->work.p, st),
       "sgemm");
    ck(launch_colsum(rows, OUT, s->dZ3.p, G + OFF_B3, st), "colsum");
    ck(launch_sgemm(false, true, rows, HID, OUT, s->dZ3.p, OUT, P + OFF_W3, OUT, s->dA.p, HID, false, 1, nullptr, st),
       "sgemm");
    ck(launch_gelu_back(rows * HID, s->dA.p, s->Z2.p, s->dZ.p, st), "gelu_back");
    ck(launch_sgemm(true, false, HID, HID, rows, s->A1.p, HID, s->dZ.p, HID, G + OFF_W2, HID, false, SPLITS,
                    s->work.p, st),
       "sgemm");
    ck(launch_colsum(rows, HID, s->dZ.p, G + OFF_B2, st), "colsum");
    ck(launch_sgemm(false, true, rows, HID, HID, s->dZ.p, HID, P + OFF_W2, HID, s->dA.p, HID, false, 1, nullptr, st),
       "sgemm");
    ck(launch_gelu_back(rows * HID, s->dA.p, s->Z1.p, s->dZ.p, st), "gelu_back");
    ck(launch_sgemm(true, false, IN, HID, rows, s->Xb.p, IN, s->dZ.p, HID, G + OFF_W1, HID, false, SPLITS, s->work.p,
                    st),
       "sgemm");
    ck(launch_colsum(rows, HID, s->dZ.p, G + OFF_B1, st), "colsum");
}

void grow_dataset(mgpu_selector* s, size_t need) {
    if (need <= s->cap) return;
    size_t cap = std::max<size_t>(need, s->cap * 2);
    cap = std::max<size_t>(cap, 1 << 16);
    DevArray<float> X;
    DevArray<uint8_t> Y;
    X.alloc(cap * sel::IN);
    Y.alloc(cap * sel::NV);
    if (s->n) {
        ck(cudaMemcpyAsync(X.p, s->X.p, s->n * sel::IN * 4, cudaMemcpyDeviceToDevice, s->stream), "D2D");
        ck(cudaMemcpyAsync(Y.p, s->Y.p, s->n * sel::NV, cudaMemcpyDeviceToDevice, s->stream), "D2D");
        ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
    }
    std::swap(s->X.p, X.p);
    std::swap(s->X.n, X.n);
    std::swap(s->Y.p, Y.p);
    std::swap(s->Y.n, Y.n);
    s->cap = cap;
}

int need_sel(const mgpu_selector* s) {
    if (!s) {
        set_error("null selector");
        return MGPU_ERR_ARG;
    }
    return MGPU_OK;
}

}  // namespace
}  // namespace mgpu

extern "C" {

int mgpu_selector_create(int device, uint64_t seed, mgpu_selector** out) {
    if (!out) {
        set_error("null argument");
        return MGPU_ERR_ARG;
    }
    *out = nullptr;
    return guarded([&] {
        DeviceGuard g(device);
        std::unique_ptr<mgpu_selector> s(new mgpu_selector());
        s->device = device;
        ck(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        s->params.assign(sel::N_PARAMS, 0.0f);
        std::mt19937_64 rng(seed);
        auto init = [&](int off, int fan_in, int count) {
            const double bound = 1.0 / std::sqrt((double)fan_in);
            std::uniform_real_distribution<double> u(-bound, bound);
            for (int i = 0; i < count; ++i) s->params[off + i] = (float)u(rng);
        };
        init(sel::OFF_W1, sel::IN, sel::IN * sel::HID);
        init(sel::OFF_W2, sel::HID, sel::HID * sel::HID);
        init(sel::OFF_W3, sel::HID, sel::HID * sel::OUT);
        s->d_params.alloc(sel::N_PARAMS);
        s->d_grad.alloc(sel::N_PARAMS);
        s->d_m.alloc(sel::N_PARAMS);
        s->d_v.alloc(sel::N_PARAMS);
        s->d_wimg.alloc(sel::WEIGHT_IMAGE_BYTES);
        s->work.alloc((size_t)SPLITS * sel::IN * sel::HID);
        s->err.alloc(1);
        upload_params(s.get());
        ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
        *out = s.release();
        return MGPU_OK;
    });
}

void mgpu_selector_destroy(mgpu_selector* s) {
    if (!s) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(s->device);
    delete s;
    if (prev >= 0) cudaSetDevice(prev);
}

int mgpu_selector_get_params(mgpu_selector* s, float* params) {
    if (int rc = need_sel(s)) return rc;
    return guarded([&] {
        if (!params) throw ArgFail("null argument");
        std::memcpy(params, s->params.data(), s->params.size() * 4);
        return MGPU_OK;
    });
}

int mgpu_selector_set_params(mgpu_selector* s, const float* params) {
    if (int rc = need_sel(s)) return rc;
    return guarded([&] {
        if (!params) throw ArgFail("null argument");
        DeviceGuard g(s->device);
        std::memcpy(s->params.data(), params, s->params.size() * 4);
        upload_params(s);
        ck(cudaMemsetAsync(s->d_m.p, 0, s->d_m.bytes(), s->stream), "cudaMemsetAsync");
        ck(cudaMemsetAsync(s->d_v.p, 0, s->d_v.bytes(), s->stream), "cudaMemsetAsync");
        s->adam_t = 0;
        ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
        return MGPU_OK;
    });
}

int mgpu_selector_dataset_size(const mgpu_selector* s, uint64_t* n) {
    if (int rc = need_sel(s)) return rc;
    if (!n) {
        set_error("null argument");
        return MGPU_ERR_ARG;
    }
    *n = s->n;
    return MGPU_OK;
}

int mgpu_selector_clear(mgpu_selector* s) {
    if (int rc = need_sel(s)) return rc;
    s->n = 0;
    return MGPU_OK;
}

int mgpu_selector_add_samples(mgpu_selector* s, const float* X, const uint8_t* Y, uint64_t n) {
    if (int rc = need_sel(s)) return rc;
    return guarded([&] {
        if ((!X || !Y) && n) throw ArgFail("null argument");
        for (uint64_t i = 0; i < n * sel::NV; ++i)
            if (Y[i] >= sel::NCLS) throw ArgFail("class label out of range");
        DeviceGuard g(s->device);
        grow_dataset(s, s->n + n);
        ck(cudaMemcpyAsync(s->X.p + s->n * sel::IN, X, n * sel::IN * 4, cudaMemcpyHostToDevice, s->stream), "H2D");
        ck(cudaMemcpyAsync(s->Y.p + s->n * sel::NV, Y, n * sel::NV, cudaMemcpyHostToDevice, s->stream), "H2D");
        ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
        s->n += n;
        return MGPU_OK;
    });
}

int mgpu_selector_get_samples(mgpu_selector* s, uint64_t first, uint64_t n, float* X, uint8_t* Y) {
    if (int rc = need_sel(s)) return rc;
    return guarded([&] {
        if (first + n > s->n) throw ArgFail("sample range outside the dataset");
        DeviceGuard g(s->device);
        if (X) ck(cudaMemcpyAsync(X, s->X.p + first * sel::IN, n * sel::IN * 4, cudaMemcpyDeviceToHost, s->stream), "D2H");
        if (Y) ck(cudaMemcpyAsync(Y, s->Y.p + first * sel::NV, n * sel::NV, cudaMemcpyDeviceToHost, s->stream), "D2H");
        ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
        return MGPU_OK;
    });
}

int mgpu_selector_harvest(mgpu_selector* s, mgpu_ctx* ctx, double keep_central, uint64_t seed, uint64_t* added) {
    if (int rc = need_sel(s)) return rc;
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (ctx->cfg.recon != MGPU_RECON_TENO || ctx->K != 10 || ctx->cfg.teno_variant == MGPU_TENO_REFERENCE ||
            ctx->single())
            throw Unsupported("harvest needs an FP64 context with corrected or robust TENO at p = 3");
        if (ctx->cfg.device != s->device) throw ArgFail("selector and context are on different devices");
        DeviceGuard g(s->device);
        // TENO decisions of the current state
        ctx->reconstruct(ctx->U.p, ctx->masks.p);
        std::vector<uint8_t> mk((size_t)ctx->N * 4);
        ck(cudaMemcpyAsync(mk.data(), ctx->masks.p, mk.size(), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        std::mt19937_64 rng(seed);
        std::uniform_real_distribution<double> u(0.0, 1.0);
        std::vector<uint32_t> cells;
        for (uint32_t c = 0; c < ctx->N; ++c) {
            const bool central = mk[4 * (size_t)c] == 1 && mk[4 * (size_t)c + 1] == 1 && mk[4 * (size_t)c + 2] == 1 &&
                                 mk[4 * (size_t)c + 3] == 1;
            const double r = u(rng);
            if (!central || r < keep_central) cells.push_back(c);
        }
        DevArray<uint32_t> dc;
        dc.upload(cells);
        grow_dataset(s, s->n + cells.size());
        ck(sel::launch_harvest(ctx->teno, false, ctx->U.p, dc.p, (uint32_t)cells.size(), ctx->masks.p,
                               s->X.p + s->n * sel::IN, s->Y.p + s->n * sel::NV, ctx->stream),
           "harvest");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        s->n += cells.size();
        if (added) *added = cells.size();
        return MGPU_OK;
    });
}

int mgpu_selector_gradient(mgpu_selector* s, const float* X, const uint8_t* Y, uint32_t n, float* grad, float* loss) {
    if (int rc = need_sel(s)) return rc;
    return guarded([&] {
        if (!X || !Y || !grad || n == 0) throw ArgFail("null or empty argument");
        DeviceGuard g(s->device);
        ensure_batch(s, n);
        ck(cudaMemcpyAsync(s->Xb.p, X, (size_t)n * sel::IN * 4, cudaMemcpyHostToDevice, s->stream), "H2D");
        ck(cudaMemcpyAsync(s->Yb.p, Y, (size_t)n * sel::NV, cudaMemcpyHostToDevice, s->stream), "H2D");
        const int nb = sel::xent_blocks((int)n);
        DevArray<float> part;
        part.alloc(nb);
        forward_backward(s, (int)n, part.p);
        std::vector<float> hp(nb);
        ck(cudaMemcpyAsync(grad, s->d_grad.p, sel::N_PARAMS * 4, cudaMemcpyDeviceToHost, s->stream), "D2H");
        ck(cudaMemcpyAsync(hp.data(), part.p, nb * 4, cudaMemcpyDeviceToHost, s->stream), "D2H");
        ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
        double tot = 0;
        for (float x : hp) tot += x;
        if (loss) *loss = (float)(tot / ((double)n * sel::NV));
        return MGPU_OK;
    });
}

int mgpu_selector_train(mgpu_selector* s, uint32_t epochs, uint32_t batch, float lr, uint64_t seed,
                        float* epoch_loss) {
    if (int rc = need_sel(s)) return rc;
    return guarded([&] {
        if (s->n == 0) throw ArgFail("empty dataset");
        if (batch == 0 || epochs == 0) throw ArgFail("batch and epochs must be positive");
        if (s->n > 0xffffffffull) throw ArgFail("dataset too large");
        DeviceGuard g(s->device);
        const uint32_t n = (uint32_t)s->n;
        const uint32_t rows_max = std::min<uint32_t>(batch, n);
        ensure_batch(s, rows_max);
        const uint32_t nbatch = (n + batch - 1) / batch;
        const int pb = sel::xent_blocks((int)rows_max);
        DevArray<float> part;
        part.alloc((size_t)nbatch * pb);
        std::vector<uint32_t> perm(n);
        std::vector<float> hp((size_t)nbatch * pb);
        for (uint32_t e = 0; e < epochs; ++e) {
            std::iota(perm.begin(), perm.end(), 0u);
            std::mt19937_64 rng(seed + e);
            for (uint32_t i = n - 1; i > 0; --i) std::swap(perm[i], perm[rng() % (i + 1)]);
            s->perm.upload(perm);
            ck(cudaMemsetAsync(part.p, 0, part.bytes(), s->stream), "cudaMemsetAsync");
            for (uint32_t b = 0; b < nbatch; ++b) {
                const uint32_t off = b * batch, rows = std::min(batch, n - off);
                ck(sel::launch_gather_rows((int)rows, s->perm.p + off, s->X.p, s->Y.p, s->Xb.p, s->Yb.p, s->stream),
                   "gather");
                forward_backward(s, (int)rows, part.p + (size_t)b * pb);
                ++s->adam_t;
                const float bc1 = 1.0f - std::pow(0.9f, (float)s->adam_t);
                const float bc2 = 1.0f - std::pow(0.999f, (float)s->adam_t);
                ck(sel::launch_adam(sel::N_PARAMS, s->d_params.p, s->d_grad.p, s->d_m.p, s->d_v.p, lr, 0.9f, 0.999f,
                                    1e-8f, bc1, bc2, s->stream),
                   "adam");
            }
            ck(cudaMemcpyAsync(hp.data(), part.p, part.bytes(), cudaMemcpyDeviceToHost, s->stream), "D2H");
            ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
            double tot = 0;
            for (float x : hp) tot += x;
            if (epoch_loss) epoch_loss[e] = (float)(tot / ((double)n * sel::NV));
        }
        download_params(s);
        s->wimg_dirty = true;
        return MGPU_OK;
    });
}

int mgpu_selector_infer(mgpu_selector* s, const float* X, uint32_t n, float thr_central, float thr_directional,
                        float* logits, uint8_t* pred) {
    if (int rc = need_sel(s)) return rc;
    return guarded([&] {
        if (!X || n == 0) throw ArgFail("null or empty argument");
        DeviceGuard g(s->device);
        refresh_image(s);
        ck(sel::mlp_prepare(), "cudaFuncSetAttribute");
        DevArray<float> dx, dl;
        DevArray<uint8_t> dp;
        dx.alloc((size_t)n * sel::IN);
        if (logits) dl.alloc((size_t)n * sel::OUT);
        if (pred) dp.alloc((size_t)n * sel::NV);
        ck(cudaMemcpyAsync(dx.p, X, (size_t)n * sel::IN * 4, cudaMemcpyHostToDevice, s->stream), "H2D");
        ck(cudaMemsetAsync(s->err.p, 0, sizeof(unsigned), s->stream), "cudaMemsetAsync");
        ck(sel::launch_mlp_rows(s->d_wimg.p, (int)n, dx.p, logits ? dl.p : nullptr, pred ? dp.p : nullptr,
                                thr_central, thr_directional, s->err.p, s->stream),
           "selector inference");
        unsigned e = 0;
        ck(cudaMemcpyAsync(&e, s->err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream), "D2H");
        if (logits) ck(cudaMemcpyAsync(logits, dl.p, (size_t)n * sel::OUT * 4, cudaMemcpyDeviceToHost, s->stream), "D2H");
        if (pred) ck(cudaMemcpyAsync(pred, dp.p, (size_t)n * sel::NV, cudaMemcpyDeviceToHost, s->stream), "D2H");
        ck(cudaStreamSynchronize(s->stream), "cudaStreamSynchronize");
        if (e) {
            set_error("selector inference: a bounded wait ran out");
            return MGPU_ERR_TIMEOUT;
        }
        return MGPU_OK;
    });
}

int mgpu_set_selector(mgpu_ctx* ctx, mgpu_selector* s, float thr_central, float thr_directional) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (!s || !(thr_central > 0.0f)) {
            ctx->sel_on = false;
            ctx->drop_graphs();
            return MGPU_OK;
        }
        if (!ctx->single() || ctx->K != 10) throw Unsupported("the learned selector drives the FP32 form at p = 3");
        if (ctx->cfg.device != s->device) throw ArgFail("selector and context are on different devices");
        if (thr_central > 1.0f) throw ArgFail("central threshold above 1");
        DeviceGuard g(s->device);
        refresh_image(s);
        ck(sel::mlp_prepare(), "cudaFuncSetAttribute");
        if (!ctx->sel_wimg.p) ctx->sel_wimg.alloc(sel::WEIGHT_IMAGE_BYTES);
        if (!ctx->pred.p) ctx->pred.alloc((size_t)ctx->N * 4);
        if (!ctx->trusted.p) ctx->trusted.alloc((size_t)ctx->N * 4);
        if (!ctx->sel_err.p) ctx->sel_err.alloc(1);
        ck(cudaMemcpy(ctx->sel_wimg.p, s->d_wimg.p, sel::WEIGHT_IMAGE_BYTES, cudaMemcpyDeviceToDevice), "D2D");
        ctx->sel_thr_central = thr_central;
        ctx->sel_thr_directional = thr_directional;
        ctx->sel_on = true;
        ctx->drop_graphs();  // the captured step no longer matches
        return MGPU_OK;
    });
}

int mgpu_set_selector_every_stage(mgpu_ctx* ctx, int every_stage) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        ctx->sel_every_stage = every_stage != 0;
        ctx->drop_graphs();
        return MGPU_OK;
    });
}

int mgpu_set_selector_interval(mgpu_ctx* ctx, uint32_t steps) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (steps == 0) throw ArgFail("the prediction interval is at least one step");
        ctx->sel_interval = steps;
        ctx->drop_graphs();
        return MGPU_OK;
    });
}

int mgpu_selector_predictions(mgpu_ctx* ctx, int raw, uint8_t* out) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (!out) throw ArgFail("null argument");
        if (!ctx->pred.p) throw ArgFail("no selector attached");
        std::vector<uint8_t> pr((size_t)ctx->N * 4);
        ck(cudaMemcpyAsync(pr.data(), raw ? ctx->pred.p : ctx->trusted.p, pr.size(), cudaMemcpyDeviceToHost,
                           ctx->stream),
           "D2H");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        for (uint32_t c = 0; c < ctx->N; ++c) std::memcpy(out + 4 * (size_t)ctx->cell_old[c], &pr[4 * (size_t)c], 4);
        return MGPU_OK;
    });
}

int mgpu_selector_stats(mgpu_ctx* ctx, uint64_t* counts) {
    if (int rc = need_ready(ctx)) return rc;
    return guarded([&] {
        if (!counts) throw ArgFail("null argument");
        if (!ctx->pred.p) throw ArgFail("no selector attached");
        std::vector<uint8_t> pr((size_t)ctx->N * 4), sm(ctx->N);
        ck(cudaMemcpyAsync(pr.data(), ctx->trusted.p, pr.size(), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
        ck(cudaMemcpyAsync(sm.data(), ctx->smask.p, sm.size(), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
        unsigned e = 0;
        ck(cudaMemcpyAsync(&e, ctx->sel_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream), "D2H");
        ck(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
        uint64_t conf_vars = 0, conf_cells = 0, evaluated = 0, full = 0;
        for (uint32_t c = 0; c < ctx->N; ++c) {
            unsigned need = 0;
            int nconf = 0;
            for (int v = 0; v < 4; ++v) {
                const unsigned p = pr[4 * (size_t)c + v], pm = p & sm[c] & 0xFu;
                const bool conf = (p & 0x80u) && pm;
                nconf += conf;
                need |= conf ? pm : sm[c];
            }
            conf_vars += nconf;
            conf_cells += nconf == 4;
            evaluated += __builtin_popcount(need);
            full += __builtin_popcount(sm[c]);
        }
        counts[0] = ctx->N;
        counts[1] = conf_cells;
        counts[2] = conf_vars;
        counts[3] = evaluated;
        counts[4] = full;
        counts[5] = e;
        return MGPU_OK;
    });
}

}  // extern "C"
