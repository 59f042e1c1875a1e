// render.cu - wavefront path tracer (placeholder until the pipeline lands).
#include "kgk_scene.h"

namespace kgk {
struct RenderState {};
void render_state_free(kgk_scene *s) {
    delete s->rs;
    s->rs = nullptr;
}
}  // namespace kgk

using namespace kgk;

extern "C" {
kgk_status kgk_render(kgk_scene *, const kgk_camera *, const kgk_camera *, const kgk_render_config *, kgk_vec *,
                      kgk_stats *) {
    return fail(KGK_ERR_UNSUPPORTED, "kgk_render: not built yet");
}
kgk_status kgk_accum_reset(kgk_scene *, int32_t, int32_t) {
    return fail(KGK_ERR_UNSUPPORTED, "kgk_accum_reset: not built yet");
}
kgk_status kgk_accum_read(kgk_scene *, double *, double *, uint64_t *) {
    return fail(KGK_ERR_UNSUPPORTED, "kgk_accum_read: not built yet");
}
kgk_status kgk_svgf(kgk_scene *, const kgk_svgf_config *, const kgk_vec *, kgk_vec *) {
    return fail(KGK_ERR_UNSUPPORTED, "kgk_svgf: not built yet");
}
kgk_status kgk_scene_load_obj(const char *, const char *, kgk_scene **) {
    return fail(KGK_ERR_UNSUPPORTED, "kgk_scene_load_obj: not built yet");
}
}
