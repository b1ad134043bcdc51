// learned_api.cpp - the C ABI of the learned rectifier (include/taa_gb300.h,
// taa_mlp_*): weight initialisation, the network alone, and training on
// records collected from resolved frames.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <new>
#include <numeric>
#include <random>
#include <vector>

#include "host_util.h"
#include "kernels.h"

using namespace taa_host;

struct taa_mlp_trainer {
    int capacity = 0;
    int sms = 0;
    void* records = nullptr;     // capacity x taa_mlp_record_t
    uint32_t* count = nullptr;   // records appended so far (may exceed the capacity)
    uint32_t* order = nullptr;   // the shuffle of the current epoch
    float* weights = nullptr;    // FP32 masters
    float* m = nullptr;          // Adam moments
    float* v = nullptr;
    float* grads = nullptr;      // gradient sums, then the loss sum and the record count
    float* partial = nullptr;    // per-CTA slabs of the same, added in CTA order
    char* blob = nullptr;
    unsigned int* status = nullptr;
    uint32_t calls = 0;          // collections so far: the first half of each record's key
};

namespace {

constexpr int kGradExtra = 2;

int record_count(taa_mlp_trainer* tr, int* n) {
    uint32_t c = 0;
    cudaError_t e = cudaMemcpy(&c, tr->count, sizeof c, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "taa_mlp: record count");
    *n = (int)std::min<uint32_t>(c, (uint32_t)tr->capacity);
    return TAA_OK;
}

int upload_weights(taa_mlp_trainer* tr, const taa_mlp_weights_t* w) {
    cudaError_t e = cudaMemcpy(tr->weights, w, sizeof *w, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = taa_dev::launch_mlp_build_blob(tr->weights, tr->blob, nullptr);
    if (e != cudaSuccess) return cuda_fail(e, "taa_mlp: weights");
    return TAA_OK;
}

}  // namespace

extern "C" {

int taa_mlp_init_weights(taa_mlp_weights_t* w, uint64_t seed, float alpha0) {
    if (!w) return fail(TAA_E_INVAL, "taa_mlp_init_weights: NULL argument");
    if (!(alpha0 > 0.f && alpha0 < 1.f)) return fail(TAA_E_INVAL, "taa_mlp_init_weights: alpha0 must be in (0, 1)");
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    std::memset(w, 0, sizeof *w);
    const float a1 = std::sqrt(6.f / (32.f + 32.f));
    for (float& x : w->w1) x = a1 * u(rng);
    for (float& x : w->w2) x = a1 * u(rng);
    for (float& x : w->w3) x = 0.01f * u(rng);
    // the constant unit's row and column are not weights
    for (int i = 0; i < 32; ++i) {
        w->w1[31 * 32 + i] = w->w1[i * 32 + 31] = 0.f;
        w->w2[31 * 32 + i] = w->w2[i * 32 + 31] = 0.f;
    }
    w->w3[31] = w->w3[32 + 31] = 0.f;
    w->b3[0] = std::log(alpha0 / (1.f - alpha0));
    w->b3[1] = 0.f;
    return TAA_OK;
}

int taa_mlp_forward(taa_ctx* c, void* stream, const float* features, float* outputs, int32_t n) {
    if (!c || !features || !outputs) return fail(TAA_E_INVAL, "taa_mlp_forward: NULL argument");
    if (!c->have_mlp) return fail(TAA_E_INVAL, "taa_mlp_forward: no weights (taa_set_mlp)");
    if (n < 0) return fail(TAA_E_INVAL, "taa_mlp_forward: n %d", n);
    if (n == 0) return TAA_OK;
    unsigned int* status = nullptr;
    cudaError_t e = taa_dev::device_status_word(&status);
    if (e == cudaSuccess) e = taa_dev::launch_mlp_forward(c->mlp_blob, features, outputs, n, status, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "taa_mlp_forward");
    return TAA_OK;
}

int taa_mlp_trainer_create(int32_t capacity, taa_mlp_trainer** out) {
    if (!out) return fail(TAA_E_INVAL, "taa_mlp_trainer_create: NULL argument");
    *out = nullptr;
    if (capacity < 128 || capacity > (1 << 26)) return fail(TAA_E_INVAL, "taa_mlp_trainer_create: capacity %d", capacity);
    if (sizeof(taa_mlp_record_t) != taa_dev::learned_record_bytes() ||
        sizeof(taa_mlp_weights_t) != sizeof(float) * (size_t)taa_dev::learned_param_count())
        return fail(TAA_E_INVAL, "taa_mlp_trainer_create: record or weight layout mismatch");
    taa_mlp_trainer* tr = new (std::nothrow) taa_mlp_trainer();
    if (!tr) return fail(TAA_E_NOMEM, "taa_mlp_trainer_create: host allocation failed");
    tr->capacity = capacity;
    const size_t np = (size_t)taa_dev::learned_param_count();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&tr->sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaMalloc(&tr->records, sizeof(taa_mlp_record_t) * (size_t)capacity);
    if (e == cudaSuccess) e = cudaMalloc(&tr->count, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&tr->order, sizeof(uint32_t) * (size_t)capacity);
    if (e == cudaSuccess) e = cudaMalloc(&tr->weights, sizeof(float) * np);
    if (e == cudaSuccess) e = cudaMalloc(&tr->m, sizeof(float) * np);
    if (e == cudaSuccess) e = cudaMalloc(&tr->v, sizeof(float) * np);
    if (e == cudaSuccess) e = cudaMalloc(&tr->grads, sizeof(float) * (np + kGradExtra));
    if (e == cudaSuccess)
        e = cudaMalloc(&tr->partial, sizeof(float) * (size_t)taa_dev::learned_grad_floats() * 2 * (size_t)tr->sms);
    if (e == cudaSuccess) e = cudaMalloc(&tr->blob, (size_t)taa_dev::learned_blob_bytes());
    if (e == cudaSuccess) e = taa_dev::device_status_word(&tr->status);
    if (e == cudaSuccess) e = cudaMemset(tr->count, 0, sizeof(uint32_t));
    if (e != cudaSuccess) {
        taa_mlp_trainer_destroy(tr);
        return e == cudaErrorMemoryAllocation ? fail(TAA_E_NOMEM, "taa_mlp_trainer_create: out of device memory")
                                              : cuda_fail(e, "taa_mlp_trainer_create");
    }
    *out = tr;
    return TAA_OK;
}

int taa_mlp_trainer_destroy(taa_mlp_trainer* tr) {
    if (!tr) return TAA_OK;
    for (void* p : {tr->records, (void*)tr->count, (void*)tr->order, (void*)tr->weights, (void*)tr->m, (void*)tr->v,
                    (void*)tr->grads, (void*)tr->partial, (void*)tr->blob})
        if (p) cudaFree(p);
    delete tr;
    return TAA_OK;
}

int taa_mlp_collect(taa_mlp_trainer* tr, taa_ctx* c, void* stream, const taa_frame_io_t* io, const void* truth,
                    size_t truth_pitch, float fraction, uint32_t seed) {
    if (!tr || !c || !io || !truth) return fail(TAA_E_INVAL, "taa_mlp_collect: NULL argument");
    if (!c->have_uniforms) return fail(TAA_E_INVAL, "taa_mlp_collect: taa_set_uniforms was not called");
    if (!(fraction >= 0.f && fraction <= 1.f)) return fail(TAA_E_INVAL, "taa_mlp_collect: fraction %g", fraction);
    const taa_desc_t& d = c->desc;
    if (truth_pitch < (size_t)d.out_width * 16 || truth_pitch % 16 || (uintptr_t)truth % 16)
        return fail(TAA_E_ALIGN, "taa_mlp_collect: truth must be RGBA32F with 16-byte aligned rows");
    int rc = learned_supported(d, c->uniforms, io, "taa_mlp_collect");
    if (rc) return rc;
    taa_dev::FrameArgs a{};
    if ((rc = frame_args(d, c->uniforms, c->cas_const1[0], io, "taa_mlp_collect", &a))) return rc;
    const taa_dev::Img t{(const char*)truth, truth_pitch, d.out_width, d.out_height};
    cudaError_t e = taa_dev::launch_resolve_learned((int)d.history_format, d.motion_format == TAA_MOTION_RGBA16F ? 4 : 2,
                                                    true, false, c->uniforms, a, nullptr, tr->records, tr->count,
                                                    (uint32_t)tr->capacity, seed, tr->calls, fraction, t,
                                                    (cudaStream_t)stream);
    if (e == cudaSuccess) ++tr->calls;
    if (e != cudaSuccess) return cuda_fail(e, "taa_mlp_collect");
    return TAA_OK;
}

int taa_mlp_record_count(taa_mlp_trainer* tr, int32_t* count) {
    if (!tr || !count) return fail(TAA_E_INVAL, "taa_mlp_record_count: NULL argument");
    int n = 0;
    int rc = record_count(tr, &n);
    if (rc) return rc;
    *count = n;
    return TAA_OK;
}

int taa_mlp_records(taa_mlp_trainer* tr, int32_t first, int32_t count, taa_mlp_record_t* out) {
    if (!tr || !out) return fail(TAA_E_INVAL, "taa_mlp_records: NULL argument");
    int n = 0;
    int rc = record_count(tr, &n);
    if (rc) return rc;
    if (first < 0 || count < 0 || first + count > n)
        return fail(TAA_E_INVAL, "taa_mlp_records: [%d, %d) outside the %d records", first, first + count, n);
    cudaError_t e = cudaMemcpy(out, (const char*)tr->records + sizeof(taa_mlp_record_t) * (size_t)first,
                               sizeof(taa_mlp_record_t) * (size_t)count, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "taa_mlp_records");
    return TAA_OK;
}

int taa_mlp_gradients(taa_mlp_trainer* tr, const taa_mlp_weights_t* w, int32_t first, int32_t count,
                      taa_mlp_weights_t* grad, float* loss_sum) {
    if (!tr || !w || !grad) return fail(TAA_E_INVAL, "taa_mlp_gradients: NULL argument");
    int n = 0;
    int rc = record_count(tr, &n);
    if (rc) return rc;
    if (first < 0 || count < 1 || first + count > n)
        return fail(TAA_E_INVAL, "taa_mlp_gradients: [%d, %d) outside the %d records", first, first + count, n);
    if ((rc = upload_weights(tr, w))) return rc;
    const size_t np = (size_t)taa_dev::learned_param_count();
    cudaError_t e = cudaMemset(tr->grads, 0, sizeof(float) * (np + kGradExtra));
    const int grid = std::max(1, std::min((count + 127) / 128, 2 * tr->sms));
    if (e == cudaSuccess)
        e = taa_dev::launch_mlp_train(tr->blob, tr->records, nullptr, first, count, tr->grads, tr->partial, tr->status,
                                      grid, nullptr);
    if (e == cudaSuccess) e = taa_dev::launch_mlp_map_grads(tr->grads, nullptr);
    std::vector<float> g(np + kGradExtra);
    if (e == cudaSuccess) e = cudaMemcpy(g.data(), tr->grads, sizeof(float) * g.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "taa_mlp_gradients");
    std::memcpy(grad, g.data(), sizeof *grad);
    if (loss_sum) *loss_sum = g[np];
    return TAA_OK;
}

int taa_mlp_train(taa_mlp_trainer* tr, taa_mlp_weights_t* w, int32_t steps, int32_t batch, float lr, uint64_t seed,
                  float* loss_first, float* loss_last) {
    if (!tr || !w) return fail(TAA_E_INVAL, "taa_mlp_train: NULL argument");
    int n = 0;
    int rc = record_count(tr, &n);
    if (rc) return rc;
    if (steps < 1 || batch < 128 || batch > n || !(lr > 0.f))
        return fail(TAA_E_INVAL, "taa_mlp_train: steps %d, batch %d (128..%d records), lr %g", steps, batch, n, lr);
    if ((rc = upload_weights(tr, w))) return rc;
    const size_t np = (size_t)taa_dev::learned_param_count();
    cudaError_t e = cudaMemset(tr->m, 0, sizeof(float) * np);
    if (e == cudaSuccess) e = cudaMemset(tr->v, 0, sizeof(float) * np);
    if (e == cudaSuccess) e = cudaMemset(tr->grads, 0, sizeof(float) * (np + kGradExtra));
    // The collection appends records in whatever order its CTAs run; the
    // epochs shuffle the records' canonical order (by key) instead, so that a
    // training run repeats bit for bit on the same collections.
    std::vector<uint32_t> keys(2 * (size_t)n), canon(n), order(n);
    if (e == cudaSuccess)
        e = cudaMemcpy2D(keys.data(), 2 * sizeof(uint32_t),
                         (const char*)tr->records + offsetof(taa_mlp_record_t, key), sizeof(taa_mlp_record_t),
                         2 * sizeof(uint32_t), (size_t)n, cudaMemcpyDeviceToHost);
    std::iota(canon.begin(), canon.end(), 0u);
    std::sort(canon.begin(), canon.end(), [&](uint32_t a, uint32_t b) {
        return keys[2 * (size_t)a] != keys[2 * (size_t)b] ? keys[2 * (size_t)a] < keys[2 * (size_t)b]
                                                        : keys[2 * (size_t)a + 1] < keys[2 * (size_t)b + 1];
    });
    std::mt19937_64 rng(seed);
    int pos = n;  // forces a shuffle before the first batch
    const int grid = std::max(1, std::min((batch + 127) / 128, 2 * tr->sms));
    for (int step = 1; step <= steps && e == cudaSuccess; ++step) {
        if (pos + batch > n) {
            std::iota(order.begin(), order.end(), 0u);
            std::shuffle(order.begin(), order.end(), rng);
            for (uint32_t& o : order) o = canon[o];
            e = cudaMemcpy(tr->order, order.data(), sizeof(uint32_t) * (size_t)n, cudaMemcpyHostToDevice);
            pos = 0;
            if (e != cudaSuccess) break;
        }
        e = taa_dev::launch_mlp_train(tr->blob, tr->records, tr->order, pos, batch, tr->grads, tr->partial, tr->status,
                                      grid, nullptr);
        pos += batch;
        if (e == cudaSuccess && (step == 1 || step == steps)) {
            float lc[2];
            e = cudaMemcpy(lc, tr->grads + np, sizeof lc, cudaMemcpyDeviceToHost);
            const float mean = lc[1] > 0.f ? lc[0] / lc[1] : 0.f;
            if (step == 1 && loss_first) *loss_first = mean;
            if (step == steps && loss_last) *loss_last = mean;
        }
        // cosine decay of the learning rate to a tenth over the run
        const float lr_t = lr * (0.1f + 0.45f * (1.f + std::cos(3.14159265f * (float)(step - 1) / (float)steps)));
        if (e == cudaSuccess)
            e = taa_dev::launch_mlp_adam(tr->weights, tr->m, tr->v, tr->grads, step, lr_t, tr->blob, nullptr);
    }
    if (e == cudaSuccess) e = cudaMemcpy(w, tr->weights, sizeof *w, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "taa_mlp_train");
    return TAA_OK;
}

}  // extern "C"
