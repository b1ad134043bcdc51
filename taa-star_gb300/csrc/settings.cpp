// settings.cpp - the .ini settings of the TAA class: writeSettingsToIni and
// readSettingsFromIni (source/taa.hpp:1198-1339) with the typed helpers of
// source/IniUtil.cpp:55-190, producing and reading text the way the INI
// library the reference vendors does (external/include/mini/ini.h: section
// and key names lower-cased, `key=value` lines, sections separated by one
// newline, ';' comment lines, the last of repeated keys wins).
//
// Host code only: no device work.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

#include "../../include/taa_gb300.h"
#include "host_util.h"

using namespace taa_host;

namespace {

// The field kinds of source/IniUtil.h (iniWriteBool, ...Bool32, ...Int, ...Float,
// ...Vec2, ...Vec4, ...IVec4).
enum class Kind { Bool, Bool32, Int, Float, Vec2, Vec4, IVec4 };

std::string lower(std::string s) {
    for (char& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

const char* const kSpace = " \t\n\r\f\v";
std::string trim(const std::string& s) {
    size_t b = s.find_first_not_of(kSpace);
    if (b == std::string::npos) return std::string();
    size_t e = s.find_last_not_of(kSpace);
    return s.substr(b, e - b + 1);
}

// std::to_string of the reference's writers (IniUtil.cpp:59-63).
std::string fmt_float(float v) {
    char b[512];
    std::snprintf(b, sizeof b, "%f", (double)v);
    return b;
}
std::string fmt_int(long v) { return std::to_string(v); }

// ------------------------------------------------------------------ writing
struct Writer {
    std::string text;
    bool first_section = true;
    bool section_has_keys = false;
    void section(const std::string& name) {
        if (!first_section) text += "\n";
        text += "[" + lower(name) + "]";
        first_section = false;
        section_has_keys = false;
    }
    void put(const std::string& key, const std::string& value) {
        text += "\n" + lower(key) + "=" + trim(value);
        section_has_keys = true;
    }
    void field(const std::string& key, Kind k, void* p) {
        static const char* const sfx[4] = {".x", ".y", ".z", ".w"};
        switch (k) {
            case Kind::Bool: put(key, *(uint32_t*)p ? "1" : "0"); break;
            case Kind::Bool32: put(key, std::to_string(*(uint32_t*)p)); break;
            case Kind::Int: put(key, fmt_int(*(int32_t*)p)); break;
            case Kind::Float: put(key, fmt_float(*(float*)p)); break;
            case Kind::Vec2:
                for (int i = 0; i < 2; ++i) put(key + sfx[i], fmt_float(((float*)p)[i]));
                break;
            case Kind::Vec4:
                for (int i = 0; i < 4; ++i) put(key + sfx[i], fmt_float(((float*)p)[i]));
                break;
            case Kind::IVec4:
                for (int i = 0; i < 4; ++i) put(key + sfx[i], fmt_int(((int32_t*)p)[i]));
                break;
        }
    }
};

// ------------------------------------------------------------------ reading
using Ini = std::map<std::string, std::map<std::string, std::string>>;

// mINI's reader: lines split at '\n' with '\r' and NUL dropped, trimmed; ';'
// starts a comment; "[name]" opens a section (text after ';' cut first);
// `key=value` splits at the first '=' not written as "\=", both sides trimmed;
// key/value lines before the first section are ignored.
Ini parse(const char* text, size_t length) {
    Ini ini;
    std::string section;
    bool in_section = false;
    size_t i = 0;
    while (i <= length) {
        std::string line;
        while (i < length && text[i] != '\n') {
            if (text[i] != '\r' && text[i] != '\0') line += text[i];
            ++i;
        }
        ++i;  // past the newline (or the end)
        line = trim(line);
        if (line.empty() || line[0] == ';') continue;
        if (line[0] == '[') {
            size_t c = line.find(';');
            if (c != std::string::npos) line = line.substr(0, c);
            size_t close = line.rfind(']');
            if (close != std::string::npos) {
                section = lower(trim(line.substr(1, close - 1)));
                ini[section];
                in_section = true;
                continue;
            }
        }
        std::string norm = line;
        for (size_t k = 0; k + 1 < norm.size(); ++k)
            if (norm[k] == '\\' && norm[k + 1] == '=') norm[k] = norm[k + 1] = ' ';
        size_t eq = norm.find('=');
        if (eq == std::string::npos || !in_section) continue;
        std::string key = trim(line.substr(0, eq));
        for (size_t k = key.find("\\="); k != std::string::npos; k = key.find("\\=", k + 1)) key.replace(k, 2, "=");
        ini[section][lower(key)] = trim(line.substr(eq + 1));
    }
    return ini;
}

struct Reader {
    const Ini& ini;
    std::string sec;
    int rc = TAA_OK;
    void section(const std::string& name) { sec = lower(name); }
    // ini[section][name] of the reference: "" when absent
    std::string get(const std::string& key) const {
        auto s = ini.find(sec);
        if (s == ini.end()) return std::string();
        auto k = s->second.find(lower(key));
        return k == s->second.end() ? std::string() : k->second;
    }
    bool bad(const std::string& key, const std::string& v) {
        if (rc == TAA_OK) rc = fail(TAA_E_INVAL, "settings: [%s] %s = '%s' is not a number", sec.c_str(), key.c_str(), v.c_str());
        return false;
    }
    // std::stoul / std::stol / std::stof: leading number, the rest ignored; no
    // number or out of range is an error
    bool read_ulong(const std::string& key, unsigned long* out) {
        std::string v = get(key);
        if (v.empty()) return false;
        errno = 0;
        char* end = nullptr;
        unsigned long r = std::strtoul(v.c_str(), &end, 10);
        if (end == v.c_str() || errno == ERANGE) return bad(key, v);
        *out = r;
        return true;
    }
    bool read_long(const std::string& key, long* out) {
        std::string v = get(key);
        if (v.empty()) return false;
        errno = 0;
        char* end = nullptr;
        long r = std::strtol(v.c_str(), &end, 10);
        if (end == v.c_str() || errno == ERANGE) return bad(key, v);
        *out = r;
        return true;
    }
    void read_float(const std::string& key, float* out) {
        std::string v = get(key);
        if (v.empty()) return;
        errno = 0;
        char* end = nullptr;
        float r = std::strtof(v.c_str(), &end);
        if (end == v.c_str() || errno == ERANGE) {
            bad(key, v);
            return;
        }
        *out = r;
    }
    void read_int(const std::string& key, int32_t* out) {
        long r;
        if (read_long(key, &r)) *out = (int32_t)r;
    }
    void field(const std::string& key, Kind k, void* p) {
        static const char* const sfx[4] = {".x", ".y", ".z", ".w"};
        switch (k) {
            case Kind::Bool: {  // IniUtil.cpp:149: "1" or "true"
                std::string v = get(key);
                if (!v.empty()) *(uint32_t*)p = (v == "1" || v == "true") ? 1u : 0u;
                break;
            }
            case Kind::Bool32: {
                unsigned long r;
                if (read_ulong(key, &r)) *(uint32_t*)p = (uint32_t)r;
                break;
            }
            case Kind::Int: read_int(key, (int32_t*)p); break;
            case Kind::Float: read_float(key, (float*)p); break;
            case Kind::Vec2:
                for (int i = 0; i < 2; ++i) read_float(key + sfx[i], (float*)p + i);
                break;
            case Kind::Vec4:
                for (int i = 0; i < 4; ++i) read_float(key + sfx[i], (float*)p + i);
                break;
            case Kind::IVec4:
                for (int i = 0; i < 4; ++i) read_int(key + sfx[i], (int32_t*)p + i);
                break;
        }
    }
};

// The members of one parameter set in the order writeSettingsToIni writes them
// (source/taa.hpp:1205-1238; readSettingsFromIni reads the same keys).
template <class V> void visit_parameters(V& v, taa_parameters_t& p) {
    v.field("mPassThrough", Kind::Bool32, &p.mPassThrough);
    v.field("mColorClampingOrClipping", Kind::Int, &p.mColorClampingOrClipping);
    v.field("mShapedNeighbourhood", Kind::Bool32, &p.mShapedNeighbourhood);
    v.field("mVarianceClipping", Kind::Bool32, &p.mVarianceClipping);
    v.field("mVarClipGamma", Kind::Float, &p.mVarClipGamma);
    v.field("mUseYCoCg", Kind::Bool32, &p.mUseYCoCg);
    v.field("mLumaWeightingLottes", Kind::Bool32, &p.mLumaWeightingLottes);
    v.field("mDepthCulling", Kind::Bool32, &p.mDepthCulling);
    v.field("mRejectOutside", Kind::Bool32, &p.mRejectOutside);
    v.field("mUnjitterNeighbourhood", Kind::Bool32, &p.mUnjitterNeighbourhood);
    v.field("mUnjitterCurrentSample", Kind::Bool32, &p.mUnjitterCurrentSample);
    v.field("mUnjitterFactor", Kind::Float, &p.mUnjitterFactor);
    v.field("mAlpha", Kind::Float, &p.mAlpha);
    v.field("mMinAlpha", Kind::Float, &p.mMinAlpha);
    v.field("mMaxAlpha", Kind::Float, &p.mMaxAlpha);
    v.field("mRejectionAlpha", Kind::Float, &p.mRejectionAlpha);
    v.field("mUseVelocityVectors", Kind::Int, &p.mUseVelocityVectors);
    v.field("mVelocitySampleMode", Kind::Int, &p.mVelocitySampleMode);
    v.field("mInterpolationMode", Kind::Int, &p.mInterpolationMode);
    v.field("mToneMapLumaKaris", Kind::Bool32, &p.mToneMapLumaKaris);
    v.field("mAddNoise", Kind::Bool32, &p.mAddNoise);
    v.field("mNoiseFactor", Kind::Float, &p.mNoiseFactor);
    v.field("mReduceBlendNearClamp", Kind::Bool32, &p.mReduceBlendNearClamp);
    v.field("mDynamicAntiGhosting", Kind::Bool32, &p.mDynamicAntiGhosting);
    v.field("mDebugMask", Kind::Vec4, &p.mDebugMask);
    v.field("mDebugMode", Kind::Int, &p.mDebugMode);
    v.field("mDebugScale", Kind::Float, &p.mDebugScale);
    v.field("mDebugCenter", Kind::Bool32, &p.mDebugCenter);
    v.field("mDebugToScreenOutput", Kind::Bool32, &p.mDebugToScreenOutput);
    v.field("mVelBasedAlpha", Kind::Bool32, &p.mVelBasedAlpha);
    v.field("mVelBasedAlphaMax", Kind::Float, &p.mVelBasedAlphaMax);
    v.field("mVelBasedAlphaFactor", Kind::Float, &p.mVelBasedAlphaFactor);
    v.field("mRayTraceAugment", Kind::Bool32, &p.mRayTraceAugment);
}

template <class V> void visit_primary(V& v, taa_settings_t& s) {
    v.section("TAA_Primary");  // source/taa.hpp:1241-1256
    v.field("mTaaEnabled", Kind::Bool, &s.mTaaEnabled);
    v.field("mSampleDistribution", Kind::Int, &s.mSampleDistribution);
    v.field("mSharpener", Kind::Int, &s.mSharpener);
    v.field("mSharpenFactor", Kind::Float, &s.mSharpenFactor);
    v.field("mSplitScreen", Kind::Bool, &s.mSplitScreen);
    v.field("mSplitX", Kind::Int, &s.mSplitX);
    v.field("mFixedJitterIndex", Kind::Int, &s.mFixedJitterIndex);
    v.field("mJitterExtraScale", Kind::Float, &s.mJitterExtraScale);
    v.field("mJitterSlowMotion", Kind::Int, &s.mJitterSlowMotion);
    v.field("mJitterRotateDegrees", Kind::Float, &s.mJitterRotateDegrees);
    v.field("mResetHistoryOnChange", Kind::Bool, &s.mResetHistoryOnChange);
}

template <class V> void visit_postprocess(V& v, taa_settings_t& s) {
    v.section("TAA_Postprocess");  // source/taa.hpp:1258-1264
    v.field("mPostProcessEnabled", Kind::Bool, &s.mPostProcessEnabled);
    v.field("zoom", Kind::Bool32, &s.zoom);
    v.field("showZoomBox", Kind::Bool32, &s.showZoomBox);
    v.field("zoomSrcLTWH", Kind::IVec4, &s.zoomSrcLTWH);
    v.field("zoomDstLTWH", Kind::IVec4, &s.zoomDstLTWH);
}

int check_count(const taa_settings_t& s, const char* who) {
    if (s.mDebugSampleOffsetsCount < 1 || s.mDebugSampleOffsetsCount > TAA_SETTINGS_MAX_SAMPLE_OFFSETS)
        return fail(TAA_E_INVAL, "%s: mDebugSampleOffsetsCount %d not in 1..%d", who, s.mDebugSampleOffsetsCount,
                    TAA_SETTINGS_MAX_SAMPLE_OFFSETS);
    return ok();
}

}  // namespace

extern "C" {

int taa_settings_default(taa_settings_t* out) {
    if (!out) return fail(TAA_E_INVAL, "taa_settings_default: NULL argument");
    std::memset(out, 0, sizeof *out);
    taa_default_parameters(&out->param[0]);
    out->param[1] = out->param[0];
    // source/taa.hpp:1350-1420
    out->mTaaEnabled = 1;
    out->mSampleDistribution = 1;
    out->mSharpener = 0;
    out->mSharpenFactor = 0.5f;
    out->mSplitScreen = 0;
    out->mSplitX = 0;
    out->mFixedJitterIndex = -1;
    out->mJitterExtraScale = 1.0f;
    out->mJitterSlowMotion = 1;
    out->mJitterRotateDegrees = 0.f;
    out->mResetHistoryOnChange = 1;
    out->mDebugSampleOffsetsCount = 1;  // { {0, 0} }
    out->mPostProcessEnabled = 1;
    // push_constants_for_postprocess (source/taa.hpp:101-111)
    out->zoom = 0;
    out->showZoomBox = 1;
    const int32_t src[4] = {960 - 10, 540 - 10, 20, 20}, dst[4] = {1920 - 200 - 10, 10, 200, 200};
    std::memcpy(out->zoomSrcLTWH, src, sizeof src);
    std::memcpy(out->zoomDstLTWH, dst, sizeof dst);
    return ok();
}

int taa_settings_write_ini(const taa_settings_t* settings, char* text, size_t capacity, size_t* length) {
    static const char* who = "taa_settings_write_ini";
    if (!settings || !length) return fail(TAA_E_INVAL, "%s: NULL argument", who);
    int rc;
    if ((rc = check_count(*settings, who))) return rc;
    taa_settings_t s = *settings;
    Writer w;
    for (int i = 0; i < 2; ++i) {
        w.section("TAA_Param_" + std::to_string(i));
        visit_parameters(w, s.param[i]);
    }
    visit_primary(w, s);
    w.field("mDebugSampleOffsets.size", Kind::Int, &s.mDebugSampleOffsetsCount);
    for (int i = 0; i < s.mDebugSampleOffsetsCount; ++i)
        w.field("mDebugSampleOffsets_" + std::to_string(i), Kind::Vec2, s.mDebugSampleOffsets[i]);
    visit_postprocess(w, s);
    *length = w.text.size();
    if (!text) return ok();
    if (capacity < w.text.size() + 1)
        return fail(TAA_E_INVAL, "%s: %zu bytes needed, capacity %zu", who, w.text.size() + 1, capacity);
    std::memcpy(text, w.text.c_str(), w.text.size() + 1);
    return ok();
}

int taa_settings_read_ini(taa_settings_t* settings, const char* text, size_t length) {
    static const char* who = "taa_settings_read_ini";
    if (!settings || (!text && length)) return fail(TAA_E_INVAL, "%s: NULL argument", who);
    int rc;
    if ((rc = check_count(*settings, who))) return rc;
    const Ini ini = parse(text ? text : "", length);
    taa_settings_t s = *settings;
    Reader r{ini};
    for (int i = 0; i < 2; ++i) {
        r.section("TAA_Param_" + std::to_string(i));
        visit_parameters(r, s.param[i]);
    }
    visit_primary(r, s);
    // source/taa.hpp:1320-1324: the list takes the stored size (at least one
    // entry, new entries zero), then the stored entries
    int32_t n = 0;
    r.read_int("mDebugSampleOffsets.size", &n);
    if (r.rc != TAA_OK) return r.rc;
    const int32_t count = n > 1 ? n : 1;
    if (count > TAA_SETTINGS_MAX_SAMPLE_OFFSETS)
        return fail(TAA_E_INVAL, "%s: %d debug sample offsets, at most %d", who, count,
                    TAA_SETTINGS_MAX_SAMPLE_OFFSETS);
    for (int i = s.mDebugSampleOffsetsCount; i < count; ++i) s.mDebugSampleOffsets[i][0] = s.mDebugSampleOffsets[i][1] = 0.f;
    s.mDebugSampleOffsetsCount = count;
    for (int i = 0; i < n; ++i) r.field("mDebugSampleOffsets_" + std::to_string(i), Kind::Vec2, s.mDebugSampleOffsets[i]);
    visit_postprocess(r, s);
    if (r.rc != TAA_OK) return r.rc;
    *settings = s;
    return ok();
}

}  // extern "C"
