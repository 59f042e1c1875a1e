// kgk_scene.h - the opaque scene handle behind kgk_scene*.
#pragma once

#include "kgk_internal.h"

namespace kgk {

// Growable device staging buffer for host-pointer arguments.
struct Staging {
    void *ptr = nullptr;
    size_t cap = 0;
    kgk_status reserve(size_t bytes);
    ~Staging();
};

struct RenderState;  // render.cu
struct NrcState;     // nrc.cu
void render_state_free(kgk_scene *s);
bool is_device_ptr(const void *p);

// SVGF history kept across frames (svgf.cu).
struct SvgfState {
    int W = 0, H = 0;
    kgk_svgf_buffer *prev = nullptr, *cur = nullptr;   // compat: reference-layout records
    float4 *hist = nullptr, *hist_prev = nullptr;      // standard: demodulated colour, w = history length
    float2 *mom = nullptr, *mom_prev = nullptr;        // standard: luminance moments
    float4 *nd = nullptr, *nd_prev = nullptr;          // standard: normal + depth, this frame and the last
    int *mat = nullptr, *mat_prev = nullptr;           // standard: material id (-1 = no hit), same
    float *gz = nullptr;                               // standard: sigma_z |grad depth|
    float4 *col = nullptr, *tmp = nullptr;             // standard: colour + variance ping-pong
    unsigned char *compat_scratch = nullptr;           // compat: the filter's scratch (compat_scratch_bytes)
    kgk_camera prev_cam{};
    bool has_prev = false;
};
void svgf_state_free(kgk_scene *s);
void nrc_state_free(kgk_scene *s);
// The G-buffer and camera of the last frame rendered with write_gbuffer=1.
bool svgf_gbuffer(kgk_scene *s, int *W, int *H, const float4 **pos, const float4 **nrm, const float4 **alb,
                  const float4 **emi, kgk_camera *cam);
// The frame the last kgk_render kept on the device (called with out == NULL).
bool render_kept_frame(kgk_scene *s, int *W, int *H, const float4 **frame);

// RGBA8 frame output (svgf.cu): two device buffers used in turn, and a copy
// stream that brings a finished one to host memory while the next frame is
// computed on the scene's stream.
struct OutputState {
    size_t npx = 0;
    uchar4 *rgba8[2] = {nullptr, nullptr};
    int slot = 0;
    cudaStream_t copy = nullptr;
    cudaEvent_t done[2] = {nullptr, nullptr}, copied[2] = {nullptr, nullptr};
};
void output_state_free(kgk_scene *s);

// save_png's tone mapping (IO_save_png.cuh:26,7,47-52) on the host:
// powf(x, 1/2.2f), clamp to [0,1], x255 truncated (NaN gives 0).
uint8_t tone_host(float x);
// Thresholds of tone_host: entry k-1 is the smallest float x >= 0 with
// tone_host(x) >= k (k = 1..255), computed once with this machine's powf, so
// a device lookup gives tone_host's bytes exactly.
const float *tone_thresholds();
// Tone-maps npx pixels on the device (in, out: device pointers) on stream st.
kgk_status tonemap_device(const float4 *in, size_t npx, uchar4 *out, cudaStream_t st);

}  // namespace kgk

struct kgk_scene {
    int device = 0;
    cudaStream_t stream = nullptr;
    kgk::DevScene dev;
    bool built = false;
    kgk::Staging staging;
    kgk::RenderState *rs = nullptr;
    kgk::SvgfState *svgf = nullptr;
    kgk::NrcState *nrc = nullptr;
    kgk::OutputState *out = nullptr;
};
