// taa.hpp - C++ mirror of the reference's taa<CF> component over the C ABI.
//
// The reference's class (source/taa.hpp:26-1427) owns the TAA images per
// frame in flight, builds the jitter, keeps the projection/view matrices of
// each frame, fills the uniform block in update() and records the dispatch
// chain in render().  This header keeps that interface - the same method
// names, parameter block and per-frame bookkeeping - for a C++ application
// that renders with CUDA: images are device buffers, "recording" is enqueuing
// on a CUDA stream, and the dispatch is taa_resolve().  GUI, .ini and
// RenderDoc parts of the reference class are not carried over.
//
// Usage, once per frame (as wookiee drives the reference, source/main.cpp:4122-4123):
//   P_jit = taa.get_jittered_projection_matrix(P, frame);   // render the G-buffer with P_jit
//   taa.save_history_proj_matrix(P, frame);
//   taa.update(view, frame, seconds);
//   taa.render(frame, stream);                             // result(frame) / sharpened(frame)
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

#include "../include/taa_gb300.h"

namespace taa_gb300 {

struct Mat4 {
    double m[16];  // column-major
    static Mat4 identity() {
        Mat4 r{};
        r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0;
        return r;
    }
};

// A pitched device image.
struct Image {
    void* ptr = nullptr;
    size_t pitch = 0;
};

inline void check(int rc) {
    if (rc < 0) throw std::runtime_error(std::string("taa: ") + taa_last_error());
}

template <size_t CF> class taa {
    static_assert(CF > 1, "the history of frame N is frame N-1's (source/taa.hpp:1005)");

   public:
    using Parameters = taa_parameters_t;

    // taa<CF>::Parameters mParameters[2] and the other settings the reference edits through its GUI
    Parameters mParameters[2];
    bool mTaaEnabled = true;
    int mSampleDistribution = 1;  // source/taa.hpp:1353
    bool mResetHistory = false;
    bool mResetHistoryOnChange = true;
    bool mSplitScreen = false;
    int mSplitX = 0;
    uint32_t mSharpener = TAA_SHARPEN_OFF;  // 0 off, 1 simple, 2 CAS
    float mSharpenFactor = 0.5f;
    taa_jitter_opts_t mJitterDebug{-1, 1, 0.f, 1.f};
    uint32_t mForm = TAA_FORM_AUTO;

    taa() {
        check(taa_default_parameters(&mParameters[0]));
        mParameters[1] = mParameters[0];
    }
    ~taa() { release(); }
    taa(const taa&) = delete;
    taa& operator=(const taa&) = delete;

    // source/taa.hpp:263-360: borrow the G-buffer images of every frame in
    // flight, create the result/history images (owned here) and the context.
    void set_source_image_views(int targetWidth, int targetHeight, int sourceWidth, int sourceHeight,
                                const std::array<Image, CF>& color, const std::array<Image, CF>& depth,
                                const std::array<Image, CF>& velocity, uint32_t motionFormat = TAA_MOTION_RGBA16F) {
        release();
        mSrcColor = color;
        mSrcDepth = depth;
        mSrcVelocity = velocity;
        mIn[0] = sourceWidth;
        mIn[1] = sourceHeight;
        mOut[0] = targetWidth;
        mOut[1] = targetHeight;
        mUpsampling = targetWidth != sourceWidth || targetHeight != sourceHeight;
        for (size_t i = 0; i < CF; ++i) {
            alloc(mResult[i], 8);
            alloc(mHistory[i], 16);
            alloc(mSharpened[i], 8);
        }
        taa_desc_t d{sizeof(taa_desc_t), sourceWidth, sourceHeight, targetWidth, targetHeight, TAA_HISTORY_RGBA32F,
                     motionFormat, mForm, mSharpener, mSharpenFactor, 0};
        check(taa_create(&d, &mCtx));
        mSplitX = targetWidth / 2;  // source/taa.hpp:354
        if (cudaEventCreate(&mT0) != cudaSuccess || cudaEventCreate(&mT1) != cudaSuccess)
            throw std::runtime_error("taa: cudaEventCreate failed");
    }

    // source/taa.hpp:150-233 (jitter in NDC; sample distributions 0..4)
    std::array<float, 2> get_jitter_offset_for_frame(uint64_t frameId, int32_t* numSamples = nullptr) const {
        std::array<float, 2> j{0.f, 0.f};
        check(taa_get_jitter_offset(mSampleDistribution, frameId, mIn[0], mIn[1], &mJitterDebug, j.data(),
                                    numSamples));
        return j;
    }

    // source/taa.hpp:243-253
    Mat4 get_jittered_projection_matrix(const Mat4& proj, uint64_t frameId) const {
        if (!mTaaEnabled) return proj;
        std::array<float, 2> j = get_jitter_offset_for_frame(frameId);
        Mat4 r = proj;
        for (int c = 0; c < 4; ++c) {
            r.m[c * 4 + 0] = proj.m[c * 4 + 0] + (double)j[0] * proj.m[c * 4 + 3];
            r.m[c * 4 + 1] = proj.m[c * 4 + 1] + (double)j[1] * proj.m[c * 4 + 3];
        }
        return r;
    }

    // source/taa.hpp:235-240: the unjittered projection of this frame
    void save_history_proj_matrix(const Mat4& proj, uint64_t frameId) { mProj[frameId % CF] = proj; }

    // source/taa.hpp:894-971: reset on parameter change (debug fields excluded),
    // jitter, time, split screen, near/far, CasSetup on sharpness change.
    void update(const Mat4& view, uint64_t frameId, double seconds, float nearPlane = 0.1f, float farPlane = 1000.f) {
        if (mResetHistoryOnChange && mOldParamsValid) {
            for (int i = 0; i < 2; ++i) {
                Parameters a = mParameters[i], b = mOldParams[i];
                for (Parameters* p : {&a, &b}) {
                    p->mDebugMode = 0;
                    p->mDebugScale = 0.f;
                    p->mDebugCenter = 0;
                    std::memset(p->mDebugMask, 0, sizeof p->mDebugMask);
                    p->mDebugToScreenOutput = 0;
                }
                if (std::memcmp(&a, &b, sizeof(Parameters)) != 0) mResetHistory = true;
            }
        }
        mView[frameId % CF] = view;
        int32_t n = 0;
        std::array<float, 2> j = get_jitter_offset_for_frame(frameId, &n);
        for (int i = 0; i < 2; ++i) {
            mUniforms.param[i] = mParameters[i];
            if (mParameters[i].mRayTraceHistoryCount < 0) mUniforms.param[i].mRayTraceHistoryCount = n;
        }
        mUniforms.mJitterNdc[0] = j[0];
        mUniforms.mJitterNdc[1] = j[1];
        mUniforms.mJitterNdc[2] = mUniforms.mJitterNdc[3] = 0.f;
        const float t = (float)seconds;
        const float f[4] = {.125f, .25f, .5f, 1.f};
        for (int i = 0; i < 4; ++i) mUniforms.mSinTime[i] = std::sin(f[i] * t);
        mUniforms.mUpsampling = mUpsampling;
        mUniforms.splitScreen = mSplitScreen;
        mUniforms.splitX = mSplitX;
        mUniforms.mBypassHistoryUpdate = 0;
        mUniforms.mResetHistory = mResetHistory;
        mUniforms.mCamNearPlane = nearPlane;
        mUniforms.mCamFarPlane = farPlane;
        if (mSharpener != mCtxSharpener || mSharpenFactor != mCtxSharpenFactor) {
            check(taa_set_sharpener(mCtx, mSharpener, mSharpenFactor));
            mCtxSharpener = mSharpener;
            mCtxSharpenFactor = mSharpenFactor;
        }
        mResetHistory = false;
        mOldParams[0] = mParameters[0];
        mOldParams[1] = mParameters[1];
        mOldParamsValid = true;
    }

    // source/taa.hpp:974-1192: the matrices of this and the previous frame in
    // FP64, then the resolve (and the fused sharpen) of frame `frameId`.
    // The very first frame has no history: the result is the source colour.
    void render(uint64_t frameId, cudaStream_t stream) {
        const size_t cur = frameId % CF, prev = (frameId + CF - 1) % CF;
        if (!mTaaEnabled || !mHaveHistory) {
            copy_source(cur, stream);
            mHaveHistory = mTaaEnabled;
            return;
        }
        check(taa_compose_matrices(mProj[cur].m, mView[cur].m, mProj[prev].m, mView[prev].m,
                                   mUniforms.mInverseViewProjMatrix, mUniforms.mHistoryViewProjMatrix));
        check(taa_set_uniforms(mCtx, &mUniforms));
        taa_frame_io_t io{};
        io.color = mSrcColor[cur].ptr;
        io.color_pitch = mSrcColor[cur].pitch;
        io.depth = mSrcDepth[cur].ptr;
        io.depth_pitch = mSrcDepth[cur].pitch;
        io.velocity = mSrcVelocity[cur].ptr;
        io.velocity_pitch = mSrcVelocity[cur].pitch;
        // the first resolved frame has no history written yet: read zeros (the
        // reference reads the uninitialised image there, taa.hpp:989-990)
        io.history = mFirstResolve ? nullptr : mHistory[prev].ptr;
        io.history_pitch = mHistory[prev].pitch;
        mFirstResolve = false;
        io.history_depth = mSrcDepth[prev].ptr;
        io.history_depth_pitch = mSrcDepth[prev].pitch;
        io.history_out = mHistory[cur].ptr;
        io.history_out_pitch = mHistory[cur].pitch;
        io.result = mResult[cur].ptr;
        io.result_pitch = mResult[cur].pitch;
        if (mSharpener != TAA_SHARPEN_OFF) {
            io.sharpened = mSharpened[cur].ptr;
            io.sharpened_pitch = mSharpened[cur].pitch;
        }
        mShowSharpened[cur] = mSharpener != TAA_SHARPEN_OFF;
        cudaEventRecord(mT0, stream);
        check(taa_resolve(mCtx, stream, &io));
        cudaEventRecord(mT1, stream);
        mTimed = true;
    }

    // source/taa.hpp:367-374: GPU time of the last resolve, in ms (waits for it)
    float duration() {
        if (!mTimed) return 0.f;
        float ms = 0.f;
        cudaEventSynchronize(mT1);
        cudaEventElapsedTime(&ms, mT0, mT1);
        return ms;
    }

    // the image to show for a frame: the sharpened one with a sharpener (taa.hpp:1137)
    const Image& result(uint64_t frameId) const {
        return mShowSharpened[frameId % CF] ? mSharpened[frameId % CF] : mResult[frameId % CF];
    }
    const Image& history(uint64_t frameId) const { return mHistory[frameId % CF]; }
    taa_ctx* context() const { return mCtx; }

   private:
    void alloc(Image& im, size_t texel) {
        if (cudaMallocPitch(&im.ptr, &im.pitch, (size_t)mOut[0] * texel, (size_t)mOut[1]) != cudaSuccess)
            throw std::runtime_error("taa: cudaMallocPitch failed");
    }
    void copy_source(size_t cur, cudaStream_t s) {
        mShowSharpened[cur] = false;  // nothing was sharpened for this frame
        if (mUpsampling) return;  // the reference blits with scaling; a headless caller reads the source itself
        cudaMemcpy2DAsync(mResult[cur].ptr, mResult[cur].pitch, mSrcColor[cur].ptr, mSrcColor[cur].pitch,
                          (size_t)mOut[0] * 8, (size_t)mOut[1], cudaMemcpyDeviceToDevice, s);
        // the first resolved frame runs with mResetHistory (alpha = 1)
        mResetHistory = true;
        mFirstResolve = true;
    }
    void release() {
        if (mCtx) taa_destroy(mCtx);
        mCtx = nullptr;
        for (size_t i = 0; i < CF; ++i)
            for (Image* im : {&mResult[i], &mHistory[i], &mSharpened[i]}) {
                if (im->ptr) cudaFree(im->ptr);
                im->ptr = nullptr;
            }
        if (mT0) cudaEventDestroy(mT0);
        if (mT1) cudaEventDestroy(mT1);
        mT0 = mT1 = nullptr;
    }

    taa_ctx* mCtx = nullptr;
    int mIn[2] = {0, 0}, mOut[2] = {0, 0};
    bool mUpsampling = false;
    std::array<Image, CF> mSrcColor{}, mSrcDepth{}, mSrcVelocity{};
    std::array<Image, CF> mResult{}, mHistory{}, mSharpened{};
    std::array<Mat4, CF> mProj{}, mView{};
    taa_uniforms_t mUniforms{};
    Parameters mOldParams[2]{};
    bool mOldParamsValid = false;
    bool mHaveHistory = false;
    bool mFirstResolve = true;
    std::array<bool, CF> mShowSharpened{};
    uint32_t mCtxSharpener = TAA_SHARPEN_OFF;
    float mCtxSharpenFactor = 0.5f;
    cudaEvent_t mT0 = nullptr, mT1 = nullptr;
    bool mTimed = false;
};

}  // namespace taa_gb300
