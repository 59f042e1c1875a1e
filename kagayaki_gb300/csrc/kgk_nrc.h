// kgk_nrc.h - radiance-cache MLP state and device entry points (nrc.cu).
#pragma once

#include "kgk_internal.h"

namespace kgk {
namespace nrc {
constexpr int kWidth = 64;      // hidden width
constexpr int kLayers = 5;      // hidden layers
constexpr int kRaw = 13;        // raw query floats: p(3, normalised) n(3) v(3) roughness albedo(3)
constexpr int kPitch = 72;      // BF16 row pitch of the shared-memory weight image
constexpr int kOutRows = 16;    // output layer rows, padded (3 live)
constexpr int kImgElems = kLayers * kWidth * kPitch + kOutRows * kPitch;
constexpr int kParams = kLayers * kWidth * kWidth + 3 * kWidth;  // 20,672
constexpr float kEpsRel = 0.01f;
constexpr float kInitScale = 128.0f;
constexpr int kScaleGrowth = 1000;
}  // namespace nrc

struct NrcState {
    kgk_nrc_config cfg{};
    float *w = nullptr, *m = nullptr, *v = nullptr, *g = nullptr;  // FP32 master weights, Adam, gradient
    unsigned short *img = nullptr;   // BF16 weight image (shared-memory layout)
    unsigned short *trH = nullptr;   // training scratch: activations H_l, [layer][row][64]
    unsigned short *trD = nullptr;   // training scratch: output gradients dZ_l, [layer][row][64]
    int tr_cap = 0;                  // rows the scratch holds
    float *scal = nullptr;           // [0] loss scale, [1] last loss
    int *ints = nullptr;             // [0] non-finite flag, [1] clean steps since the last scale change,
                                     // [2] inference timeout flag
    int step = 0;
    int sms = 0;
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
