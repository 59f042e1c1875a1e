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
void render_state_free(kgk_scene *s);
bool is_device_ptr(const void *p);

}  // namespace kgk

struct kgk_scene {
    int device = 0;
    cudaStream_t stream = nullptr;
    kgk::DevScene dev;
    bool built = false;
    kgk::Staging staging;
    kgk::RenderState *rs = nullptr;
};
