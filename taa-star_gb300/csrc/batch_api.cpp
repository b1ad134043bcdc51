// batch_api.cpp - the batch C ABI (include/taa_gb300.h, taa_batch_*): many
// views of any size resolved by one persistent launch of the tiled FP32 form,
// with per-view arguments in device slots and a tile shape and job order
// chosen by measurement (taa_batch_autotune).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

#include "host_util.h"
#include "kernels.h"

using taa_dev::BatchKey;
using taa_dev::BatchShapeInfo;
using taa_dev::BatchView;
using namespace taa_host;

namespace {

constexpr size_t kMapBytes = sizeof(CUtensorMap);  // 128, 64-byte aligned

// Byte layout of one argument slot: views | tensor maps [shape][view] | tma_ok [shape][view].
struct SlotLayout {
    size_t views, maps, ok, total;
    explicit SlotLayout(int n) {
        views = 0;
        maps = (sizeof(BatchView) * (size_t)n + 127) / 128 * 128;
        ok = maps + kMapBytes * (size_t)n * taa_dev::kBatchShapes;
        total = (ok + sizeof(int) * (size_t)n * taa_dev::kBatchShapes + 255) / 256 * 256;
    }
};

const int kShapeDims[taa_dev::kBatchShapes][2] = {{32, 8}, {16, 16}, {32, 16}, {16, 8}, {8, 8}, {32, 16}};

// The shape id of a tuning: the exact tiles by size, or the fast strips.
int shape_id(int w, int h, int form) {
    if (form == TAA_FORM_FAST) return w == 32 && h == 16 ? taa_dev::kBatchFastShape : -1;
    if (form != 0 && form != TAA_FORM_TILED) return -1;
    for (int i = 0; i < taa_dev::kBatchFastShape; ++i)
        if (kShapeDims[i][0] == w && kShapeDims[i][1] == h) return i;
    return -1;
}

}  // namespace

struct taa_batch {
    int n = 0;
    int device = 0, sms = 0;
    std::vector<taa_desc_t> desc;
    std::vector<taa_uniforms_t> uniforms;
    std::vector<char> have_uniforms;
    SlotLayout layout{1};
    char* d_slots = nullptr;                 // TAA_BATCH_SLOTS x layout.total
    char* h_slots = nullptr;                 // pinned staging of the same size
    cudaEvent_t slot_copied[TAA_BATCH_SLOTS] = {};
    bool slot_ready[TAA_BATCH_SLOTS] = {};
    BatchKey slot_key[TAA_BATCH_SLOTS] = {};
    uint32_t* d_jobs = nullptr;              // the active job list
    size_t jobs_cap = 0;
    int njobs = 0;
    taa_batch_tuning_t tuning{32, 8, TAA_SCHEDULE_LARGEST_FIRST, 0, 0.f, TAA_FORM_TILED};
    bool fast_ok = false;                    // created with TAA_FORM_AUTO / TAA_FORM_FAST: the strips may run
};

namespace {

// The job list of a tile shape and schedule: (view, tile x, tile y) triples.
std::vector<uint32_t> make_jobs(const taa_batch& b, int tw, int th, int schedule) {
    const int n = b.n;
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    auto tiles = [&](int v) {
        const taa_desc_t& d = b.desc[v];
        return std::make_pair((d.out_width + tw - 1) / tw, (d.out_height + th - 1) / th);
    };
    if (schedule == TAA_SCHEDULE_LARGEST_FIRST)
        std::stable_sort(order.begin(), order.end(), [&](int p, int q) {
            return (long long)b.desc[p].out_width * b.desc[p].out_height >
                   (long long)b.desc[q].out_width * b.desc[q].out_height;
        });
    std::vector<uint32_t> jobs;
    if (schedule == TAA_SCHEDULE_INTERLEAVED) {
        std::vector<int> next(n, 0);
        bool any = true;
        while (any) {
            any = false;
            for (int v : order) {
                auto [tx, ty] = tiles(v);
                if (next[v] < tx * ty) {
                    jobs.push_back(taa_dev::make_job(v, next[v] % tx, next[v] / tx));
                    ++next[v];
                    any = true;
                }
            }
        }
    } else {
        for (int v : order) {
            auto [tx, ty] = tiles(v);
            for (int y = 0; y < ty; ++y)
                for (int x = 0; x < tx; ++x) jobs.push_back(taa_dev::make_job(v, x, y));
        }
    }
    return jobs;
}

size_t max_jobs(const taa_batch& b) {
    size_t m = 0;
    for (int s = 0; s < taa_dev::kBatchShapes; ++s) {
        size_t t = 0;
        for (const taa_desc_t& d : b.desc)
            t += (size_t)((d.out_width + kShapeDims[s][0] - 1) / kShapeDims[s][0]) *
                 (size_t)((d.out_height + kShapeDims[s][1] - 1) / kShapeDims[s][1]);
        m = std::max(m, t);
    }
    return m;
}

int upload_jobs(taa_batch& b, const taa_batch_tuning_t& t, cudaStream_t s) {
    std::vector<uint32_t> jobs = make_jobs(b, t.tile_w, t.tile_h, t.schedule);
    if (jobs.size() > b.jobs_cap) return fail(TAA_E_INVAL, "taa_batch: job list larger than its buffer");
    cudaError_t e = cudaMemcpyAsync(b.d_jobs, jobs.data(), jobs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host vector goes out of scope
    if (e != cudaSuccess) return cuda_fail(e, "taa_batch: job list upload");
    b.njobs = (int)jobs.size();
    return TAA_OK;
}

int check_tuning(const taa_batch& b, const taa_batch_tuning_t& t) {
    if (shape_id(t.tile_w, t.tile_h, t.form) < 0)
        return fail(TAA_E_INVAL,
                    "taa_batch: tile shape %dx%d (form %d) is not one of 32x8, 16x16, 32x16, 16x8, 8x8 (TILED) or "
                    "32x16 (FAST)",
                    t.tile_w, t.tile_h, t.form);
    if (t.form == TAA_FORM_FAST && !b.fast_ok)
        return fail(TAA_E_UNSUPPORTED, "taa_batch: the batch was created with TAA_FORM_TILED");
    if (t.schedule < TAA_SCHEDULE_VIEW_ORDER || t.schedule > TAA_SCHEDULE_INTERLEAVED)
        return fail(TAA_E_INVAL, "taa_batch: schedule %d", t.schedule);
    if (t.ctas_per_sm < TAA_BATCH_CTA_PER_TILE || t.ctas_per_sm > 32)
        return fail(TAA_E_INVAL, "taa_batch: ctas_per_sm %d", t.ctas_per_sm);
    return TAA_OK;
}

int grid_of(const taa_batch& b, const BatchKey& k, int ctas_per_sm, int* grid) {
    int occ = 0;
    cudaError_t e = taa_dev::batch_occupancy(k, &occ);
    if (e != cudaSuccess) return cuda_fail(e, "taa_batch: occupancy");
    if (occ < 1) return fail(TAA_E_UNSUPPORTED, "taa_batch: tile kernel does not fit on an SM");
    if (ctas_per_sm == TAA_BATCH_CTA_PER_TILE) *grid = std::max(1, b.njobs);
    else *grid = b.sms * (ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ);
    return TAA_OK;
}

int launch_slot(taa_batch& b, cudaStream_t s, int slot, const taa_batch_tuning_t& t) {
    BatchKey k = b.slot_key[slot];
    k.shape = shape_id(t.tile_w, t.tile_h, t.form);
    if (k.shape == taa_dev::kBatchFastShape && !k.hot)
        return fail(TAA_E_UNSUPPORTED, "taa_batch_launch: the fast strips run the benchmark mode only");
    int grid = 0;
    int rc = grid_of(b, k, t.ctas_per_sm, &grid);
    if (rc) return rc;
    const char* base = b.d_slots + (size_t)slot * b.layout.total;
    const BatchView* views = reinterpret_cast<const BatchView*>(base + b.layout.views);
    const CUtensorMap* maps = reinterpret_cast<const CUtensorMap*>(base + b.layout.maps) + (size_t)k.shape * b.n;
    const int* ok = reinterpret_cast<const int*>(base + b.layout.ok) + (size_t)k.shape * b.n;
    cudaError_t e = taa_dev::launch_batch(k, views, maps, ok, b.d_jobs, b.njobs, grid, s);
    if (e != cudaSuccess) return cuda_fail(e, "taa_batch_launch");
    return TAA_OK;
}

}  // namespace

extern "C" {

int taa_batch_create(const taa_desc_t* descs, int32_t n, taa_batch** out) {
    if (!descs || !out) return fail(TAA_E_INVAL, "taa_batch_create: NULL argument");
    *out = nullptr;
    if (n < 1 || n > TAA_BATCH_MAX_VIEWS) return fail(TAA_E_INVAL, "taa_batch_create: %d views (1..%d)", n, TAA_BATCH_MAX_VIEWS);
    for (int v = 0; v < n; ++v) {
        const taa_desc_t& d = descs[v];
        int rc = check_desc(d, "taa_batch_create");
        if (rc) return rc;
        if (d.history_format != TAA_HISTORY_RGBA32F)
            return fail(TAA_E_UNSUPPORTED, "taa_batch_create: view %d: batches keep RGBA32F history", v);
        if (d.motion_format != descs[0].motion_format)
            return fail(TAA_E_UNSUPPORTED, "taa_batch_create: view %d: all views share one motion format", v);
        if (d.in_width != d.out_width || d.in_height != d.out_height)
            return fail(TAA_E_UNSUPPORTED, "taa_batch_create: view %d: upsampling runs with taa_resolve", v);
        if (d.sharpener != TAA_SHARPEN_OFF)
            return fail(TAA_E_UNSUPPORTED, "taa_batch_create: view %d: sharpening runs with taa_resolve", v);
        if (d.form != TAA_FORM_AUTO && d.form != TAA_FORM_TILED && d.form != TAA_FORM_FAST)
            return fail(TAA_E_UNSUPPORTED, "taa_batch_create: view %d: batches run the tiled or fast FP32 forms", v);
        if (d.form == TAA_FORM_TILED && descs[0].form != TAA_FORM_TILED)
            return fail(TAA_E_UNSUPPORTED, "taa_batch_create: view %d: all views or none ask for TAA_FORM_TILED", v);
        if (d.flags) return fail(TAA_E_UNSUPPORTED, "taa_batch_create: view %d: flags 0x%x", v, d.flags);
        if ((d.out_width + 7) / 8 > 4096 || (d.out_height + 7) / 8 > 4096)
            return fail(TAA_E_INVAL, "taa_batch_create: view %d too large for the job encoding", v);
    }
    taa_batch* b = new (std::nothrow) taa_batch();
    if (!b) return fail(TAA_E_NOMEM, "taa_batch_create: host allocation failed");
    b->n = n;
    b->desc.assign(descs, descs + n);
    b->uniforms.resize(n);
    b->have_uniforms.assign(n, 0);
    b->layout = SlotLayout(n);
    b->fast_ok = descs[0].form != TAA_FORM_TILED;
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_slots, b->layout.total * TAA_BATCH_SLOTS);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_slots, b->layout.total * TAA_BATCH_SLOTS);
    b->jobs_cap = max_jobs(*b);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_jobs, b->jobs_cap * sizeof(uint32_t));
    for (int i = 0; i < TAA_BATCH_SLOTS && e == cudaSuccess; ++i)
        e = cudaEventCreateWithFlags(&b->slot_copied[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        taa_batch_destroy(b);
        return e == cudaErrorMemoryAllocation ? fail(TAA_E_NOMEM, "taa_batch_create: out of memory")
                                              : cuda_fail(e, "taa_batch_create");
    }
    std::memset(b->h_slots, 0, b->layout.total * TAA_BATCH_SLOTS);
    int rc = upload_jobs(*b, b->tuning, nullptr);
    if (rc) {
        taa_batch_destroy(b);
        return rc;
    }
    *out = b;
    return TAA_OK;
}

int taa_batch_destroy(taa_batch* b) {
    if (!b) return TAA_OK;
    for (cudaEvent_t ev : b->slot_copied)
        if (ev) cudaEventDestroy(ev);
    if (b->d_slots) cudaFree(b->d_slots);
    if (b->h_slots) cudaFreeHost(b->h_slots);
    if (b->d_jobs) cudaFree(b->d_jobs);
    delete b;
    return TAA_OK;
}

int taa_batch_set_uniforms(taa_batch* b, int32_t view, const taa_uniforms_t* u) {
    if (!b || !u) return fail(TAA_E_INVAL, "taa_batch_set_uniforms: NULL argument");
    if (view < 0 || view >= b->n) return fail(TAA_E_INVAL, "taa_batch_set_uniforms: view %d of %d", view, b->n);
    int rc = check_uniforms(*u, "taa_batch_set_uniforms");
    if (rc) return rc;
    b->uniforms[view] = *u;
    b->have_uniforms[view] = 1;
    return TAA_OK;
}

int taa_batch_prepare(taa_batch* b, void* stream, int32_t slot, const taa_frame_io_t* ios) {
    if (!b || !ios) return fail(TAA_E_INVAL, "taa_batch_prepare: NULL argument");
    if (slot < 0 || slot >= TAA_BATCH_SLOTS) return fail(TAA_E_INVAL, "taa_batch_prepare: slot %d", slot);
    const int n = b->n;
    BatchKey key{0, 0, b->desc[0].motion_format == TAA_MOTION_RGBA16F ? 4 : 2, 0, 0};
    for (int v = 0; v < n; ++v) {
        if (!b->have_uniforms[v]) return fail(TAA_E_INVAL, "taa_batch_prepare: view %d has no uniforms", v);
        const taa_desc_t& d = b->desc[v];
        const taa_uniforms_t& U = b->uniforms[v];
        if (!taa_dev::fast_path_supported(U, d.in_width, d.in_height, d.out_width, d.out_height, false, true))
            return fail(TAA_E_UNSUPPORTED, "taa_batch_prepare: view %d: its parameters need the plain form", v);
        const int interp = U.param[0].mInterpolationMode, hot = taa_dev::hot_parameters(U.param[0]) ? 1 : 0;
        if (interp != 0 && interp != 2)
            return fail(TAA_E_UNSUPPORTED, "taa_batch_prepare: view %d: interpolation mode %d", v, interp);
        if (v == 0) {
            key.interp = interp;
            key.hot = hot;
        } else if (interp != key.interp || hot != key.hot) {
            return fail(TAA_E_UNSUPPORTED, "taa_batch_prepare: view %d: all views share one interpolation and mode", v);
        }
        if (ios[v].debug || ios[v].segmask || ios[v].sharpened)
            return fail(TAA_E_UNSUPPORTED, "taa_batch_prepare: view %d: debug, segmask and sharpened run with taa_resolve",
                        v);
    }
    // the slot's staging may still be in a previous copy
    cudaError_t e = cudaEventSynchronize(b->slot_copied[slot]);
    if (e != cudaSuccess) return cuda_fail(e, "taa_batch_prepare: wait for the slot");
    char* h = b->h_slots + (size_t)slot * b->layout.total;
    BatchView* hv = reinterpret_cast<BatchView*>(h + b->layout.views);
    CUtensorMap* hm = reinterpret_cast<CUtensorMap*>(h + b->layout.maps);
    int* hok = reinterpret_cast<int*>(h + b->layout.ok);
    for (int v = 0; v < n; ++v) {
        hv[v].U = b->uniforms[v];
        int rc = frame_args(b->desc[v], b->uniforms[v], 0u, &ios[v], "taa_batch_prepare", &hv[v].a);
        if (rc) return rc;
        for (int s = 0; s < taa_dev::kBatchShapes; ++s) {
            BatchShapeInfo info{};
            taa_dev::batch_shape_info(s, 0, &info);
            const taa_dev::Img& hi = hv[v].a.history;
            CUtensorMap& m = hm[(size_t)s * n + v];
            std::memset(&m, 0, sizeof m);
            // the fast strips copy rows as runs of floats (2-D map), the exact tiles texel by texel (3-D)
            const int fmt = s == taa_dev::kBatchFastShape ? 2 : 0;
            hok[(size_t)s * n + v] = key.interp != 1 && hi.p && hi.w >= info.win_w && hi.h >= info.win_h &&
                                     taa_dev::encode_history_map(hi, fmt, info.win_w, info.win_h, &m);
        }
    }
    cudaStream_t s = (cudaStream_t)stream;
    e = cudaMemcpyAsync(b->d_slots + (size_t)slot * b->layout.total, h, b->layout.total, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaEventRecord(b->slot_copied[slot], s);
    if (e != cudaSuccess) return cuda_fail(e, "taa_batch_prepare: upload");
    b->slot_key[slot] = key;
    b->slot_ready[slot] = true;
    return TAA_OK;
}

int taa_batch_launch(taa_batch* b, void* stream, int32_t slot) {
    if (!b) return fail(TAA_E_INVAL, "taa_batch_launch: NULL batch");
    if (slot < 0 || slot >= TAA_BATCH_SLOTS || !b->slot_ready[slot])
        return fail(TAA_E_INVAL, "taa_batch_launch: slot %d was not prepared", slot);
    return launch_slot(*b, (cudaStream_t)stream, slot, b->tuning);
}

int taa_batch_get_tuning(const taa_batch* b, taa_batch_tuning_t* out) {
    if (!b || !out) return fail(TAA_E_INVAL, "taa_batch_get_tuning: NULL argument");
    *out = b->tuning;
    return TAA_OK;
}

int taa_batch_set_tuning(taa_batch* b, const taa_batch_tuning_t* t) {
    if (!b || !t) return fail(TAA_E_INVAL, "taa_batch_set_tuning: NULL argument");
    int rc = check_tuning(*b, *t);
    if (rc) return rc;
    rc = upload_jobs(*b, *t, nullptr);
    if (rc) return rc;
    b->tuning = *t;
    return TAA_OK;
}

int taa_batch_autotune(taa_batch* b, void* stream, int32_t slot, int32_t reps, taa_batch_tuning_t* best) {
    if (!b) return fail(TAA_E_INVAL, "taa_batch_autotune: NULL batch");
    if (slot < 0 || slot >= TAA_BATCH_SLOTS || !b->slot_ready[slot])
        return fail(TAA_E_INVAL, "taa_batch_autotune: slot %d was not prepared", slot);
    if (reps < 1 || reps > 1000) return fail(TAA_E_INVAL, "taa_batch_autotune: reps %d (1..1000)", reps);
    cudaStream_t s = (cudaStream_t)stream;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaError_t e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    if (e != cudaSuccess) return cuda_fail(e, "taa_batch_autotune: events");
    // every candidate (tile shape x job order x grid), timed in three interleaved
    // rounds; a candidate's time is its best round (a round disturbed by a clock
    // change or another job on the device does not decide the choice)
    std::vector<taa_batch_tuning_t> cands;
    for (int sh = 0; sh < taa_dev::kBatchShapes; ++sh) {
        const bool fast = sh == taa_dev::kBatchFastShape;
        if (fast && !(b->fast_ok && b->slot_key[slot].hot)) continue;
        for (int cand = 0; cand < 6; ++cand) {
            const int sched = cand % 3, grid_mode = cand < 3 ? 0 : TAA_BATCH_CTA_PER_TILE;
            cands.push_back(taa_batch_tuning_t{kShapeDims[sh][0], kShapeDims[sh][1], sched, grid_mode, -1.f,
                                               fast ? (int32_t)TAA_FORM_FAST : (int32_t)TAA_FORM_TILED});
        }
    }
    constexpr int kRounds = 3;
    int rc = TAA_OK;
    for (int round = 0; round < kRounds && rc == TAA_OK; ++round) {
        for (taa_batch_tuning_t& t : cands) {
            if ((rc = upload_jobs(*b, t, s))) break;
            if ((rc = launch_slot(*b, s, slot, t))) break;  // warm-up
            e = cudaEventRecord(t0, s);
            for (int r = 0; r < reps && e == cudaSuccess && rc == TAA_OK; ++r) rc = launch_slot(*b, s, slot, t);
            if (e == cudaSuccess) e = cudaEventRecord(t1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(t1);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t0, t1);
            if (e != cudaSuccess) {
                rc = cuda_fail(e, "taa_batch_autotune: timing");
                break;
            }
            const float per = ms / (float)reps;
            if (t.ms < 0.f || per < t.ms) t.ms = per;
        }
    }
    taa_batch_tuning_t win{};
    win.ms = -1.f;
    for (const taa_batch_tuning_t& t : cands)
        if (t.ms >= 0.f && (win.ms < 0.f || t.ms < win.ms)) win = t;
    if (rc == TAA_OK && win.ms < 0.f) rc = fail(TAA_E_INVAL, "taa_batch_autotune: no candidate ran");
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (rc == TAA_OK) rc = upload_jobs(*b, win, s);
    if (rc != TAA_OK) {
        upload_jobs(*b, b->tuning, s);  // back to the previous job list
        return rc;
    }
    b->tuning = win;
    if (best) *best = win;
    return TAA_OK;
}

}  // extern "C"
