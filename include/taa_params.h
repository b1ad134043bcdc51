/*
 * taa_params.h - the TAA parameter block and per-frame uniform block.
 *
 * These two structs are byte-identical to the blocks the reference host
 * hands to its resolve shader, so a caller that already fills them can
 * pass them through unchanged:
 *
 *   taa_parameters_t  <->  taa<CF>::Parameters        source/taa.hpp:30-77
 *                          struct Parameters (std140)  shaders/taa.comp:50-95
 *   taa_uniforms_t    <->  taa<CF>::uniforms_for_taa   source/taa.hpp:113-129
 *                          uniform Matrices  (std140)  shaders/taa.comp:102-118
 *
 * Every field is 4 bytes (VkBool32 -> uint32_t, glm::mat4 -> float[16]
 * column-major, glm::vec4 -> float[4]), so the std140 layout and the plain
 * C layout coincide: Parameters is 176 bytes with mDebugMask at offset 144,
 * uniforms_for_taa is 544 bytes with param[2] at 128, mJitterNdc at 480 and
 * splitScreen at 512.  The static asserts below pin that.
 *
 * Field names are kept identical to the reference so that presets and
 * settings written for it map one-to-one.
 */
#ifndef TAA_PARAMS_H
#define TAA_PARAMS_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Segmentation-mask / ray-trace-augment flag bits (shaders/shader_cpu_common.h:32-41). */
#define TAA_RTFLAG_OUT 0x0001u
#define TAA_RTFLAG_DIS 0x0002u
#define TAA_RTFLAG_NRM 0x0004u
#define TAA_RTFLAG_DPT 0x0008u
#define TAA_RTFLAG_MID 0x0010u
#define TAA_RTFLAG_LUM 0x0020u
#define TAA_RTFLAG_CNT 0x0040u
#define TAA_RTFLAG_ALL 0x0080u
#define TAA_RTFLAG_FXD 0x0100u
#define TAA_RTFLAG_FXA 0x0200u

/* Per-parameter-set block (source/taa.hpp:30-77). */
typedef struct taa_parameters_t {
    float    mAlpha;                    /*   0 */
    int32_t  mColorClampingOrClipping;  /*   4  0 off, 1 clamp, 2 clip-fast, 3 clip-slow */
    uint32_t mDepthCulling;             /*   8 */
    uint32_t mUnjitterNeighbourhood;    /*  12 */
    uint32_t mUnjitterCurrentSample;    /*  16 */
    float    mUnjitterFactor;           /*  20 */
    uint32_t mPassThrough;              /*  24 */
    uint32_t mUseYCoCg;                 /*  28 */
    uint32_t mShrinkChromaAxis;         /*  32 */
    uint32_t mVarianceClipping;         /*  36 */
    uint32_t mShapedNeighbourhood;      /*  40 */
    uint32_t mLumaWeightingLottes;      /*  44 */
    float    mVarClipGamma;             /*  48 */
    float    mMinAlpha;                 /*  52 */
    float    mMaxAlpha;                 /*  56 */
    float    mRejectionAlpha;           /*  60 */
    uint32_t mRejectOutside;            /*  64 */
    int32_t  mUseVelocityVectors;       /*  68  0 off, 1 movers only, 2 everything */
    int32_t  mVelocitySampleMode;       /*  72  0 simple, 1 3x3 longest, 2 3x3 closest */
    int32_t  mInterpolationMode;        /*  76  0 bilinear, 1 "b-spline", 2 Catmull-Rom */
    uint32_t mToneMapLumaKaris;         /*  80 */
    uint32_t mAddNoise;                 /*  84 */
    float    mNoiseFactor;              /*  88 */
    uint32_t mReduceBlendNearClamp;     /*  92 */
    uint32_t mDynamicAntiGhosting;      /*  96 */
    uint32_t mVelBasedAlpha;            /* 100 */
    float    mVelBasedAlphaMax;         /* 104 */
    float    mVelBasedAlphaFactor;      /* 108 */
    uint32_t mRayTraceAugment;          /* 112 */
    uint32_t mRayTraceAugmentFlags;     /* 116 */
    float    mRayTraceAugment_WNrm;     /* 120 */
    float    mRayTraceAugment_WDpt;     /* 124 */
    float    mRayTraceAugment_WMId;     /* 128 */
    float    mRayTraceAugment_WLum;     /* 132 */
    float    mRayTraceAugment_Thresh;   /* 136 */
    int32_t  mRayTraceHistoryCount;     /* 140 */
    float    mDebugMask[4];             /* 144 */
    int32_t  mDebugMode;                /* 160 */
    float    mDebugScale;               /* 164 */
    uint32_t mDebugCenter;              /* 168 */
    uint32_t mDebugToScreenOutput;      /* 172 */
} taa_parameters_t;

/* Per-frame uniform block (source/taa.hpp:113-129). */
typedef struct taa_uniforms_t {
    float            mHistoryViewProjMatrix[16]; /*   0  column-major */
    float            mInverseViewProjMatrix[16]; /*  64  column-major */
    taa_parameters_t param[2];                   /* 128  [1] is used right of splitX when splitScreen */
    float            mJitterNdc[4];              /* 480  only .xy used, NDC units */
    float            mSinTime[4];                /* 496  sin(t/8), sin(t/4), sin(t/2), sin(t) */
    uint32_t         splitScreen;                /* 512 */
    int32_t          splitX;                     /* 516 */
    uint32_t         mUpsampling;                /* 520 */
    uint32_t         mBypassHistoryUpdate;       /* 524 */
    uint32_t         mResetHistory;              /* 528 */
    float            mCamNearPlane;              /* 532 */
    float            mCamFarPlane;               /* 536 */
    float            pad1;                       /* 540 */
} taa_uniforms_t;

#ifdef __cplusplus
} /* extern "C" */
#define TAA_STATIC_ASSERT(c, m) static_assert(c, m)
#else
#define TAA_STATIC_ASSERT(c, m) _Static_assert(c, m)
#endif

TAA_STATIC_ASSERT(sizeof(taa_parameters_t) == 176, "Parameters must be 176 bytes");
TAA_STATIC_ASSERT(offsetof(taa_parameters_t, mDebugMask) == 144, "mDebugMask offset");
TAA_STATIC_ASSERT(offsetof(taa_parameters_t, mRayTraceHistoryCount) == 140, "mRayTraceHistoryCount offset");
TAA_STATIC_ASSERT(sizeof(taa_uniforms_t) == 544, "uniforms_for_taa must be 544 bytes");
TAA_STATIC_ASSERT(offsetof(taa_uniforms_t, param) == 128, "param[2] offset");
TAA_STATIC_ASSERT(offsetof(taa_uniforms_t, mJitterNdc) == 480, "mJitterNdc offset");
TAA_STATIC_ASSERT(offsetof(taa_uniforms_t, splitScreen) == 512, "splitScreen offset");
TAA_STATIC_ASSERT(offsetof(taa_uniforms_t, mCamFarPlane) == 536, "mCamFarPlane offset");

#endif /* TAA_PARAMS_H */
