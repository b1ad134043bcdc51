// synth.cu - GPU renderer of the analytic scene (taa_synth.h), FP32.
#include "kernels.h"
#include "synth_scene.h"

namespace taa_dev {
namespace {

// The sphere table travels by value in the kernel parameters (12 KB), so a
// render needs no device allocation and can be captured in a graph.
struct SphereTable {
    float v[TAA_SYNTH_MAX_SPHERES * TAA_SYNTH_SPHERE_FLOATS];
};

__global__ void __launch_bounds__(256) synth_kernel(const taa_synth_scene_t s, const SphereTable table, int frame,
                                                    const taa_synth_frame_t o) {
    __shared__ float sph[TAA_SYNTH_MAX_SPHERES * TAA_SYNTH_SPHERE_FLOATS];
    const int n = s.num_spheres * TAA_SYNTH_SPHERE_FLOATS;
    for (int i = threadIdx.y * blockDim.x + threadIdx.x; i < n; i += blockDim.x * blockDim.y) sph[i] = table.v[i];
    __syncthreads();
    int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= s.width || y >= s.height) return;

    float jx, jy;
    taa_synth::jitter_px(s, frame, jx, jy);
    float sx = (float)x + 0.5f - jx, sy = (float)y + 0.5f - jy;
    taa_synth::Hit<float> h = taa_synth::shade<float>(s, sph, frame, sx, sy);
    float r = h.r, g = h.g, b = h.b;
    uint32_t u1, u2;
    taa_synth::pixel_hash(s.seed, x, y, frame, u1, u2);
    if ((float)u1 * (1.0f / 16777216.0f) < s.firefly_fraction) {
        float f = 4.0f + (s.firefly_max - 4.0f) * ((float)u2 * (1.0f / 16777216.0f));
        r = g = b = f;
    }
    if (o.color) *texel_ptr_w<uint2>(ImgW{(char*)o.color, o.color_pitch}, x, y) = float4_to_half4(make_float4(r, g, b, 1.f));
    if (o.depth) *texel_ptr_w<float>(ImgW{(char*)o.depth, o.depth_pitch}, x, y) = h.depth;
    if (o.motion) {
        float mu = h.mx / (float)s.width, mv = h.my / (float)s.height;
        ImgW m{(char*)o.motion, o.motion_pitch};
        if (o.motion_channels == 4) {
            *texel_ptr_w<uint2>(m, x, y) = float4_to_half4(make_float4(mu, mv, 0.f, (float)h.id));
        } else {
            __half2 v = __floats2half2_rn(mu, mv);
            *texel_ptr_w<__half2>(m, x, y) = v;
        }
    }
    if (o.truth) {
        float ar = 0.f, ag = 0.f, ab = 0.f;
        for (int j = 0; j < 8; ++j)
            for (int i = 0; i < 8; ++i) {
                taa_synth::Hit<float> t =
                    taa_synth::shade<float>(s, sph, frame, (float)x + (i + 0.5f) * 0.125f, (float)y + (j + 0.5f) * 0.125f);
                ar += t.r;
                ag += t.g;
                ab += t.b;
            }
        *texel_ptr_w<float4>(ImgW{(char*)o.truth, o.truth_pitch}, x, y) =
            make_float4(ar * (1.f / 64.f), ag * (1.f / 64.f), ab * (1.f / 64.f), 1.f);
    }
}

}  // namespace

cudaError_t launch_synth(const taa_synth_scene_t& s, const float* host_spheres, int frame, const taa_synth_frame_t& out,
                         cudaStream_t stream) {
    static_assert(sizeof(SphereTable) + sizeof(taa_synth_scene_t) + sizeof(taa_synth_frame_t) + 8 < 32000,
                  "kernel parameter space");
    SphereTable t{};
    for (int i = 0; i < s.num_spheres * TAA_SYNTH_SPHERE_FLOATS; ++i) t.v[i] = host_spheres[i];
    dim3 block(32, 8), grid((s.width + 31) / 32, (s.height + 7) / 8);
    synth_kernel<<<grid, block, 0, stream>>>(s, t, frame, out);
    return cudaGetLastError();
}

}  // namespace taa_dev
