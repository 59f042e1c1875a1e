// kgk_nrc.h - radiance-cache MLP state and device entry points (nrc.cu).
#pragma once

#include "kgk_internal.h"

namespace kgk {
namespace nrc {
constexpr int kIn = 64;         // encoded input features
constexpr int kLayers = 5;      // hidden layers (ReLU): kIn -> W, then 4 x (W -> W)
constexpr int kRaw = 13;        // raw query floats: p(3, normalised) n(3) v(3) roughness albedo(3)
constexpr int kOutRows = 16;    // output layer rows, padded (3 live)

// Sizes of the network of hidden width W (64 or 128).  Master weights, FP32,
// layer by layer, each (out, in) row-major: W x 64, 4 x (W x W), 3 x W.
template <int W>
struct Net {
    static constexpr int kPitch = W + 8;  // BF16 row pitch of the shared-memory weight image
    static constexpr int kImg = kLayers * W * kPitch + kOutRows * kPitch;  // image elements
    static constexpr int kParams = W * kIn + (kLayers - 1) * W * W + 3 * W;
    // inputs of layer l (l == kLayers: the output layer)
    __host__ __device__ static constexpr int in(int l) { return l == 0 ? kIn : W; }
    // offset of layer l in the master weights
    __host__ __device__ static constexpr int woff(int l) { return l == 0 ? 0 : W * kIn + (l - 1) * W * W; }
};
static_assert(Net<64>::kParams == 20672 && Net<128>::kParams == 74112, "network sizes");

inline bool width_ok(int w) { return w == 64 || w == 128; }
inline int params_of(int w) { return w == 128 ? Net<128>::kParams : Net<64>::kParams; }
inline int img_elems_of(int w) { return w == 128 ? Net<128>::kImg : Net<64>::kImg; }
constexpr float kEpsRel = 0.01f;
constexpr float kInitScale = 128.0f;
constexpr int kScaleGrowth = 1000;
}  // namespace nrc

struct NrcState {
    kgk_nrc_config cfg{};
    float *w = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;  // FP32 master weights, Adam, gradient
    unsigned short *img = nullptr;   // BF16 weight image (shared-memory layout)
    unsigned short *trH = nullptr;   // training scratch: activations H_l, [layer][row][width]
    unsigned short *trD = nullptr;   // training scratch: output gradients dZ_l, [layer][row][width]
    int tr_cap = 0;                  // rows the scratch holds
    float *scal = nullptr;           // [0] loss scale, [1] last loss
    int *ints = nullptr;             // [0] non-finite flag, [1] clean steps since the last scale change,
                                     // [2] inference timeout flag
    int step = 0;
    int sms = 0;
    int params = 0;                  // master weights (20,672 at width 64, 74,112 at 128)
    bool ready = false;
};

kgk_status nrc_init(NrcState &N, const kgk_nrc_config *cfg, int device);
void nrc_free(NrcState &N);
// Inference on query records of `stride` floats (raw[13] first).  out: n x 3
// (may be null); rad: when non-null, rad[path] += T * max(y, 0) with T at
// floats 13..15 and the path id (int bits) at float 16 of each record.
kgk_status nrc_infer_dev(NrcState &N, const float *raw, int stride, int n, const int *n_dev, float *out, float4 *rad,
                         cudaStream_t st);
// KGK_ERR_DEVICE_CHECK (and clears the flag) when an inference kernel gave up
// a bounded wait; synchronous.
kgk_status nrc_check_error(NrcState &N);
// Gradient of the mean relative-L2 loss (times the loss scale) into N.g.
kgk_status nrc_grad_dev(NrcState &N, const float *raw, int raw_stride, const float *tgt, int tgt_stride, int n,
                        const int *n_dev, cudaStream_t st);
// Adam step from N.g (skipped when the gradient is not finite).
kgk_status nrc_step_dev(NrcState &N, cudaStream_t st);

NrcState *nrc_state(kgk_scene *s);
void nrc_state_free(kgk_scene *s);

}  // namespace kgk
