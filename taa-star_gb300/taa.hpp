// taa.hpp - C++ mirror of the reference's taa<CF> component over the C ABI.
//
// The reference's class (source/taa.hpp:26-1427) owns the TAA images per
// frame in flight, builds the jitter, keeps the projection/view matrices of
// each frame, fills the uniform block in update() and records the dispatch
// chain in render().  This header keeps that interface - the same method
// names, parameter block and per-frame bookkeeping - for a C++ application
// that renders with CUDA: images are device buffers, "recording" is enqueuing
// on a CUDA stream, and the dispatches are taa_resolve(), taa_fxaa(),
// taa_sharpen() and taa_post_process().  The settings file
// (writeSettingsToIni/readSettingsFromIni) is text in and out; the GUI and
// RenderDoc parts of the reference class are not carried over.
//
// Usage, once per frame (as wookiee drives the reference, source/main.cpp:4122-4123):
//   P_jit = taa.get_jittered_projection_matrix(P, frame);   // render the G-buffer with P_jit
//   taa.save_history_proj_matrix(P, frame);
//   taa.update(view, frame, seconds);
//   taa.render(frame, stream);                             // result(frame): the last pass's image
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

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
    taa_jitter_opts_t mJitterDebug{-1, 1, 0.f, 1.f};  // mFixedJitterIndex, mJitterSlowMotion, ...
    std::vector<std::array<float, 2>> mDebugSampleOffsets{{0.f, 0.f}};  // sample distribution 5, in pixels
    uint32_t mForm = TAA_FORM_AUTO;
    // push_constants_for_fxaa (source/taa.hpp:93-98; the reciprocal frame size is derived per call)
    taa_fxaa_params_t mFxaaPushConstants{0.75f, 0.116f, 0.0833f};
    // post-processing (source/taa.hpp:101-111, 1352): split line, zoom box and inset, debug image per side
    bool mPostProcessEnabled = true;
    struct PostProcessSettings {
        uint32_t zoom = 0, showZoomBox = 1;
        int32_t zoomSrcLTWH[4] = {960 - 10, 540 - 10, 20, 20};
        int32_t zoomDstLTWH[4] = {1920 - 200 - 10, 10, 200, 200};
    } mPostProcessPushConstants;

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
            alloc(mTemp[i], 8);
            alloc(mSegMask[i], 4);
            alloc(mDebug[i], 8);
            alloc(mPost[i], 8);
        }
        taa_desc_t d{sizeof(taa_desc_t), sourceWidth, sourceHeight, targetWidth, targetHeight, TAA_HISTORY_RGBA32F,
                     motionFormat, mForm, mSharpener, mSharpenFactor, TAA_FLAG_FXAA};
        check(taa_create(&d, &mCtx));
        mCtxSharpener = mSharpener;
        mCtxSharpenFactor = mSharpenFactor;
        mSplitX = targetWidth / 2;  // source/taa.hpp:354
        taa_post_process_params_t pp;  // the zoom boxes for this size (source/taa.hpp:355-359)
        check(taa_post_process_default_params(targetWidth, targetHeight, &pp));
        std::memcpy(mPostProcessPushConstants.zoomSrcLTWH, pp.zoom_src_ltwh, sizeof pp.zoom_src_ltwh);
        std::memcpy(mPostProcessPushConstants.zoomDstLTWH, pp.zoom_dst_ltwh, sizeof pp.zoom_dst_ltwh);
        if (cudaEventCreate(&mT0) != cudaSuccess || cudaEventCreate(&mT1) != cudaSuccess)
            throw std::runtime_error("taa: cudaEventCreate failed");
    }

    // source/taa.hpp:150-233 (jitter in NDC; sample distributions 0..4)
    std::array<float, 2> get_jitter_offset_for_frame(uint64_t frameId, int32_t* numSamples = nullptr) const {
        std::array<float, 2> j{0.f, 0.f};
        if (mSampleDistribution == 5) {  // the debug sample offsets (source/taa.hpp:207-211)
            check(taa_get_jitter_offset_custom(reinterpret_cast<const float(*)[2]>(mDebugSampleOffsets.data()),
                                               (int32_t)mDebugSampleOffsets.size(), frameId, mIn[0], mIn[1],
                                               &mJitterDebug, j.data()));
            if (numSamples) *numSamples = (int32_t)mDebugSampleOffsets.size();
            return j;
        }
        check(taa_get_jitter_offset(mSampleDistribution, frameId, mIn[0], mIn[1], &mJitterDebug, j.data(),
                                    numSamples));
        return j;
    }

    // source/taa.hpp:1344: the ray-trace-assist path runs for either active parameter set
    bool needRayTraceAssist() const {
        return mParameters[0].mRayTraceAugment || (mSplitScreen && mParameters[1].mRayTraceAugment);
    }

    // source/taa.hpp:1198-1265: the settings as .ini text (sections TAA_Param_0/1,
    // TAA_Primary, TAA_Postprocess), written as the reference writes them.
    std::string writeSettingsToIni() const {
        taa_settings_t st = settings();
        size_t n = 0;
        check(taa_settings_write_ini(&st, nullptr, 0, &n));
        std::string text(n + 1, '\0');
        check(taa_settings_write_ini(&st, &text[0], text.size(), &n));
        text.resize(n);
        return text;
    }

    // source/taa.hpp:1267-1339: read the keys present in .ini text (a whole
    // settings file of the reference, or writeSettingsToIni's output).
    void readSettingsFromIni(const std::string& text) {
        taa_settings_t st = settings();
        check(taa_settings_read_ini(&st, text.data(), text.size()));
        mParameters[0] = st.param[0];
        mParameters[1] = st.param[1];
        mTaaEnabled = st.mTaaEnabled != 0;
        mSampleDistribution = st.mSampleDistribution;
        mSharpener = (uint32_t)st.mSharpener;
        mSharpenFactor = st.mSharpenFactor;
        mSplitScreen = st.mSplitScreen != 0;
        mSplitX = st.mSplitX;
        mJitterDebug = taa_jitter_opts_t{st.mFixedJitterIndex, st.mJitterSlowMotion, st.mJitterRotateDegrees,
                                         st.mJitterExtraScale};
        mResetHistoryOnChange = st.mResetHistoryOnChange != 0;
        mDebugSampleOffsets.assign((size_t)st.mDebugSampleOffsetsCount, {0.f, 0.f});
        for (int32_t i = 0; i < st.mDebugSampleOffsetsCount; ++i)
            mDebugSampleOffsets[i] = {st.mDebugSampleOffsets[i][0], st.mDebugSampleOffsets[i][1]};
        mPostProcessEnabled = st.mPostProcessEnabled != 0;
        mPostProcessPushConstants.zoom = st.zoom;
        mPostProcessPushConstants.showZoomBox = st.showZoomBox;
        std::memcpy(mPostProcessPushConstants.zoomSrcLTWH, st.zoomSrcLTWH, sizeof st.zoomSrcLTWH);
        std::memcpy(mPostProcessPushConstants.zoomDstLTWH, st.zoomDstLTWH, sizeof st.zoomDstLTWH);
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
        // with FXAA on the segmentation mask the sharpener reads the FXAA output
        // (source/taa.hpp:1111-1139 after 1063-1104): it runs as its own pass then
        const uint32_t FXA = TAA_RTFLAG_FXA;
        mFxaa = needRayTraceAssist() &&
                ((mParameters[0].mRayTraceAugmentFlags & FXA) || (mSplitScreen && (mParameters[1].mRayTraceAugmentFlags & FXA)));
        const uint32_t fused = mFxaa ? TAA_SHARPEN_OFF : mSharpener;
        if (fused != mCtxSharpener || mSharpenFactor != mCtxSharpenFactor) {
            check(taa_set_sharpener(mCtx, fused, mSharpenFactor));
            mCtxSharpener = fused;
            mCtxSharpenFactor = mSharpenFactor;
        }
        mResetHistory = false;
        mOldParams[0] = mParameters[0];
        mOldParams[1] = mParameters[1];
        mOldParamsValid = true;
    }

    // source/taa.hpp:974-1192: the matrices of this and the previous frame in
    // FP64, then the resolve (and the sharpen pass) of frame `frameId`; on the
    // ray-trace-assist path the resolve also writes the segmentation mask, and
    // with its FXAA flag the FXAA pass and then the sharpener follow; last the
    // post-process pass when enabled (it reads the resolve's debug image when
    // a side of the split shows it).
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
        if (needRayTraceAssist()) {
            io.segmask = mSegMask[cur].ptr;
            io.segmask_pitch = mSegMask[cur].pitch;
            if (mHaveSegMask) {  // binding 12: the previous frame's mask
                io.prev_segmask = mSegMask[prev].ptr;
                io.prev_segmask_pitch = mSegMask[prev].pitch;
            }
        }
        if (mCtxSharpener != TAA_SHARPEN_OFF) {
            io.sharpened = mSharpened[cur].ptr;
            io.sharpened_pitch = mSharpened[cur].pitch;
        }
        const bool showDebug = mPostProcessEnabled && (mParameters[0].mDebugToScreenOutput ||
                                                       (mSplitScreen && mParameters[1].mDebugToScreenOutput));
        if (showDebug) {  // binding 6 (the reference writes it every frame)
            io.debug = mDebug[cur].ptr;
            io.debug_pitch = mDebug[cur].pitch;
        }
        mShown[cur] = mSharpener != TAA_SHARPEN_OFF ? Shown::Sharpened : Shown::Result;
        cudaEventRecord(mT0, stream);
        check(taa_resolve(mCtx, stream, &io));
        if (mFxaa) {
            check(taa_fxaa(mCtx, stream, mResult[cur].ptr, mResult[cur].pitch, mSegMask[cur].ptr, mSegMask[cur].pitch,
                           mTemp[cur].ptr, mTemp[cur].pitch, mOut[0], mOut[1], &mFxaaPushConstants));
            mShown[cur] = Shown::Temp;
            if (mSharpener != TAA_SHARPEN_OFF) {
                check(taa_sharpen(stream, mSharpener, mSharpenFactor, mTemp[cur].ptr, mTemp[cur].pitch,
                                  mSharpened[cur].ptr, mSharpened[cur].pitch, mOut[0], mOut[1]));
                mShown[cur] = Shown::Sharpened;
            }
        }
        if (mPostProcessEnabled) {  // source/taa.hpp:1141-1158, from the last pass's image
            const Image& last = result(frameId);
            taa_post_process_params_t pp;
            check(taa_post_process_default_params(mOut[0], mOut[1], &pp));
            std::memcpy(pp.zoom_src_ltwh, mPostProcessPushConstants.zoomSrcLTWH, sizeof pp.zoom_src_ltwh);
            std::memcpy(pp.zoom_dst_ltwh, mPostProcessPushConstants.zoomDstLTWH, sizeof pp.zoom_dst_ltwh);
            pp.zoom = mPostProcessPushConstants.zoom;
            pp.show_zoom_box = mPostProcessPushConstants.showZoomBox;
            pp.split_x = mSplitScreen ? mSplitX : -1;  // source/taa.hpp:955-959
            std::memcpy(pp.debug_l_mask, mParameters[0].mDebugMask, sizeof pp.debug_l_mask);
            std::memcpy(pp.debug_r_mask, mParameters[1].mDebugMask, sizeof pp.debug_r_mask);
            pp.debug_l_show = showDebug && mParameters[0].mDebugToScreenOutput;
            pp.debug_r_show = showDebug && mParameters[1].mDebugToScreenOutput;
            check(taa_post_process(stream, &pp, last.ptr, last.pitch, showDebug ? mDebug[cur].ptr : nullptr,
                                   mDebug[cur].pitch, mPost[cur].ptr, mPost[cur].pitch, mOut[0], mOut[1]));
            mShown[cur] = Shown::Post;
        }
        mHaveSegMask = needRayTraceAssist();
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

    // the image to show for a frame: the last pass's output (pLastProducedImageView_t, taa.hpp:1029-1137)
    const Image& result(uint64_t frameId) const {
        switch (mShown[frameId % CF]) {
            case Shown::Sharpened: return mSharpened[frameId % CF];
            case Shown::Temp: return mTemp[frameId % CF];
            case Shown::Post: return mPost[frameId % CF];
            default: return mResult[frameId % CF];
        }
    }
    const Image& history(uint64_t frameId) const { return mHistory[frameId % CF]; }
    const Image& segmentation_mask(uint64_t frameId) const { return mSegMask[frameId % CF]; }  // taa.hpp:1341
    const Image& debug_image(uint64_t frameId) const { return mDebug[frameId % CF]; }
    taa_ctx* context() const { return mCtx; }

   private:
    void alloc(Image& im, size_t texel) {
        if (cudaMallocPitch(&im.ptr, &im.pitch, (size_t)mOut[0] * texel, (size_t)mOut[1]) != cudaSuccess)
            throw std::runtime_error("taa: cudaMallocPitch failed");
    }
    enum class Shown { Result, Sharpened, Temp, Post };

    // the members the settings file holds
    taa_settings_t settings() const {
        taa_settings_t st;
        check(taa_settings_default(&st));
        st.param[0] = mParameters[0];
        st.param[1] = mParameters[1];
        st.mTaaEnabled = mTaaEnabled;
        st.mSampleDistribution = mSampleDistribution;
        st.mSharpener = (int32_t)mSharpener;
        st.mSharpenFactor = mSharpenFactor;
        st.mSplitScreen = mSplitScreen;
        st.mSplitX = mSplitX;
        st.mFixedJitterIndex = mJitterDebug.fixed_index;
        st.mJitterExtraScale = mJitterDebug.extra_scale;
        st.mJitterSlowMotion = mJitterDebug.slow_motion;
        st.mJitterRotateDegrees = mJitterDebug.rotate_degrees;
        st.mResetHistoryOnChange = mResetHistoryOnChange;
        if (mDebugSampleOffsets.empty() || mDebugSampleOffsets.size() > TAA_SETTINGS_MAX_SAMPLE_OFFSETS)
            throw std::runtime_error("taa: 1..TAA_SETTINGS_MAX_SAMPLE_OFFSETS debug sample offsets");
        st.mDebugSampleOffsetsCount = (int32_t)mDebugSampleOffsets.size();
        for (size_t i = 0; i < mDebugSampleOffsets.size(); ++i) {
            st.mDebugSampleOffsets[i][0] = mDebugSampleOffsets[i][0];
            st.mDebugSampleOffsets[i][1] = mDebugSampleOffsets[i][1];
        }
        st.mPostProcessEnabled = mPostProcessEnabled;
        st.zoom = mPostProcessPushConstants.zoom;
        st.showZoomBox = mPostProcessPushConstants.showZoomBox;
        std::memcpy(st.zoomSrcLTWH, mPostProcessPushConstants.zoomSrcLTWH, sizeof st.zoomSrcLTWH);
        std::memcpy(st.zoomDstLTWH, mPostProcessPushConstants.zoomDstLTWH, sizeof st.zoomDstLTWH);
        return st;
    }

    void copy_source(size_t cur, cudaStream_t s) {
        mShown[cur] = Shown::Result;  // nothing was sharpened for this frame
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
            for (Image* im : {&mResult[i], &mHistory[i], &mSharpened[i], &mTemp[i], &mSegMask[i], &mDebug[i], &mPost[i]}) {
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
    std::array<Image, CF> mResult{}, mHistory{}, mSharpened{}, mTemp{}, mSegMask{}, mDebug{}, mPost{};
    std::array<Mat4, CF> mProj{}, mView{};
    taa_uniforms_t mUniforms{};
    Parameters mOldParams[2]{};
    bool mOldParamsValid = false;
    bool mHaveHistory = false;
    bool mFirstResolve = true;
    std::array<Shown, CF> mShown{};
    bool mFxaa = false;
    bool mHaveSegMask = false;
    uint32_t mCtxSharpener = TAA_SHARPEN_OFF;
    float mCtxSharpenFactor = 0.5f;
    cudaEvent_t mT0 = nullptr, mT1 = nullptr;
    bool mTimed = false;
};

}  // namespace taa_gb300
