/*
 * ref_entry.cpp - runs the reference's own render-path source on the CPU.
 * TEST INFRASTRUCTURE ONLY: built by oracle/Makefile (target `ref`) from the
 * reference headers where they lie, into oracle/_ref/.  It checks the oracle
 * restatement and generates golden fixtures; nothing in the product links it.
 *
 * Exposed (extern "C"):
 *   ref_trace_closest  construct_BVH (ConstructBVH.cuh:204) + the reference
 *                      traversal willIntersectWithTriangle_nonRecursive
 *                      (ConstructBVH.cuh:286-368) for a ray set.
 *   ref_render         render() (render.cuh:21-49) over all pixels but pixel
 *                      0 (whose seed divides by zero, render.cuh:29), for a
 *                      number of frames with the persistent randSeeds.
 *   ref_svgf           ApplySVGF (SVGF.cuh:495-522) with one host thread per
 *                      pixel and __syncthreads() bound to a std::barrier over
 *                      all of them: the race-free reading of the filter.
 *   ref_disney_eval    evaluate_Disney_BRDF / _pdf (Disney_BRDF.cuh:118-183).
 *   ref_camera_setup   Camera_SetUpCamera (struct_Camera.cuh:27-35).
 *   ref_light_cdf      calculate_Lss / calculate_Lss_HDR.
 *   ref_load_obj       load_object (IO_load_WavefrontObj.cuh:10-127).
 *   ref_tinyobj_parse  tinyobjloader's raw parse, as load_object configures it.
 *   ref_load_image     stbi_loadf.
 *   ref_save_png_bytes save_png's bytes for an image (written, read back).
 *   ref_export_scene   a scene, its reference BVH and light CDF in a file
 *                      for the reference's GPU render (oracle/ref_gpu.py).
 *
 * The traversal-call counter replaces struct_stack.cuh (a 37-line fixed-size
 * stack) with an equivalent class whose constructor counts one ray per
 * traversal call; the traversal itself is the reference's.
 */
#include <atomic>
#include <chrono>
#include <barrier>
#include <thread>

#include "ref_shim.h"

// Equivalent of struct_stack.cuh with a per-thread traversal counter.
#define CUDA_MYPT_STRUCT_STACK_CUH
static thread_local long long tl_traversals = 0;
template <class T, int N> class stack {
    T buf[N];
    int idx;
public:
    stack() : idx(-1) { ++tl_traversals; }
    T &top() { return buf[idx]; }
    void push(T const &v) { buf[++idx] = v; }
    T pop() { return buf[idx--]; }
    bool full() { return idx == (N - 1); }
    bool empty() { return idx == -1; }
};

#include "struct_Camera.cuh"
#include "struct_Xorshift.cuh"
#include "NextEventEstimation.cuh"
#include "render.cuh"
#include "FileIO/IO_load_WavefrontObj.cuh"
#include "FileIO/IO_save_png.cuh"

#include <unistd.h>

thread_local kgk_uint3_ blockIdx, threadIdx, blockDim;
static std::barrier<> *g_barrier = nullptr;
void __syncthreads() {
    if (g_barrier) g_barrier->arrive_and_wait();
}

static_assert(sizeof(Vec) == 16, "Vec");
static_assert(sizeof(Triangle) == 156, "Triangle");
static_assert(sizeof(Material) == 96, "Material");
static_assert(sizeof(Camera) == 72, "Camera");
static_assert(sizeof(Texture) == 24, "Texture");
static_assert(sizeof(Ray) == 40, "Ray");

static std::vector<BVH_node_Device> g_tree;
static std::vector<Texture> g_textures;
static Texture g_hdr;

template <class F> static void parallel_for(long long n, int nthreads, F f) {
    if (nthreads <= 1) {
        for (long long i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<long long> next{0};
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; ++k)
        th.emplace_back([&] {
            for (;;) {
                long long i0 = next.fetch_add(64);
                if (i0 >= n) break;
                long long i1 = std::min(n, i0 + 64);
                for (long long i = i0; i < i1; ++i) f(i);
            }
        });
    for (auto &t : th) t.join();
}

static void release_tree() {
    for (auto &nd : g_tree)
        if (nd.face_list) (std::free)(nd.face_list);
    g_tree.clear();
}

// Loads the scene into the reference's globals and runs its BVH build.
static void load_scene(const Triangle *tris, int n, const Material *mats, int nm) {
    HOST_ObjectsData.assign(tris, tris + n);
    HOST_MaterialsData.assign(mats, mats + nm);
    ObjectsNum = n;
    HOST_BVH_tree.clear();
    construct_BVH();
    release_tree();
    g_tree.resize(HOST_BVH_tree.size());
    BVH_node_Device *dev = g_tree.data();
    Convert_BVHTreeFromHostToDevice(HOST_BVH_tree, dev);
}

extern "C" {

/* Builds the reference BVH and traces n rays.  ok[i] = the traversal's
 * return value (false on a miss or on table/stack overflow).  Returns the
 * node count of the reference tree; *traversals = number of traversal calls. */
long long ref_trace_closest(const Triangle *tris, int n, const Ray *rays, long long nrays,
                            int *face_id, float *t, unsigned char *ok, int nthreads,
                            double *build_seconds) {
    auto t0 = std::chrono::steady_clock::now();
    load_scene(tris, n, nullptr, 0);
    auto t1 = std::chrono::steady_clock::now();
    if (build_seconds) *build_seconds = std::chrono::duration<double>(t1 - t0).count();
    const BVH_node_Device *tree = g_tree.data();
    parallel_for(nrays, nthreads, [&](long long i) {
        Intersection isect;
        bool r = willIntersectWithTriangle_nonRecursive(rays[i], &isect, ObjectsNum, HOST_ObjectsData.data(), tree);
        face_id[i] = isect.face_id;
        t[i] = isect.hitpoint.distance;
        ok[i] = r ? 1 : 0;
    });
    return (long long)g_tree.size();
}

/* Leaf statistics of the reference tree built by the last ref_trace_closest
 * call: out[0] = nodes, out[1] = leaves, out[2] = max leaf size. */
void ref_bvh_stats(long long *out) {
    long long leaves = 0, maxleaf = 0;
    for (size_t i = (size_t)ObjectsNum; i < HOST_BVH_tree.size(); ++i) {
        if (HOST_BVH_tree[i].children.first == -1) {
            ++leaves;
            maxleaf = std::max<long long>(maxleaf, (long long)HOST_BVH_tree[i].face_list.size());
        }
    }
    out[0] = (long long)HOST_BVH_tree.size();
    out[1] = leaves;
    out[2] = maxleaf;
}

/* Renders `frames` frames of width x height with the reference's render().
 * out = frames * width * height * 3 floats (pixel 0 is left NaN).  gbuf (may
 * be null) receives the final frame's SVGFBuffer array (112 B per pixel).
 * textures: n_tex Texture structs with host pixel pointers.  hdr_pixels may
 * be null (no environment: background (1,1,1)).  Returns traversal calls. */
long long ref_render(const Triangle *tris, int n, const Material *mats, int nm,
                     const Texture *textures, int n_tex,
                     const float *hdr_pixels, int hdr_w, int hdr_h, int hdr_bpp,
                     const Camera *cam, const Camera *prev_cam, int width, int height, int frames,
                     int nthreads, float *out, void *gbuf) {
    load_scene(tris, n, mats, nm);
    g_textures.assign(textures, textures + n_tex);
    HOST_Light_strength_sum.clear();
    HOST_Light_strength_sum_HDR.clear();
    HOST_Exists_NoLight = false;
    calculate_Lss();
    g_hdr = Texture();
    if (hdr_pixels) {
        g_hdr.pixels = const_cast<float *>(hdr_pixels);
        g_hdr.width = hdr_w;
        g_hdr.height = hdr_h;
        g_hdr.bpp = hdr_bpp;
    }
    HOST_HDRData = &g_hdr;
    if (hdr_pixels) calculate_Lss_HDR();
    Exists_NoLight = HOST_Exists_NoLight;
    Exists_NoHDR = hdr_pixels == nullptr;
    Light_strength_sum_size = (int)HOST_Light_strength_sum.size();
    Light_strength_sum_HDR_size = (int)HOST_Light_strength_sum_HDR.size();
    image_sizeX_device = width;
    image_sizeY_device = height;
    const long long npx = (long long)width * height;
    std::memset(randSeeds, 0, sizeof(unsigned long long) * (size_t)npx);
    SVGFBuffer *sv = (SVGFBuffer *)std::calloc((size_t)npx, sizeof(SVGFBuffer));
    Vec *result = (Vec *)std::calloc((size_t)npx, sizeof(Vec));
    Camera c = *cam;
    Camera pc = prev_cam ? *prev_cam : *cam;
    // NextEventEstimation_PathTracing.cuh:18-19 reads Objects[-1] when its ray
    // misses.  A zeroed guard triangle (material 0, non-emissive) in front of
    // the array makes that read defined: the branch returns.
    std::vector<Triangle> guarded(HOST_ObjectsData.size() + 1);
    std::copy(HOST_ObjectsData.begin(), HOST_ObjectsData.end(), guarded.begin() + 1);
    const Triangle *objects = guarded.data() + 1;
    std::atomic<long long> traversals{0};
    for (int f = 0; f < frames; ++f) {
        parallel_for(npx - 1, nthreads, [&](long long i) {
            long long pos = i + 1;
            blockDim.x = 256;
            blockIdx.x = (unsigned)(pos / 256);
            threadIdx.x = (unsigned)(pos % 256);
            long long before = tl_traversals;
            render(&pc, &c, result, const_cast<Triangle *>(objects), HOST_MaterialsData.data(),
                   g_textures.data(), g_tree.data(), HOST_Light_strength_sum.data(),
                   HOST_Light_strength_sum_HDR.data(), &g_hdr, sv, 0, 0);
            traversals += tl_traversals - before;
        });
        float *o = out + (size_t)f * npx * 3;
        o[0] = o[1] = o[2] = NAN;
        for (long long p = 1; p < npx; ++p) {
            o[3 * p + 0] = result[p].x;
            o[3 * p + 1] = result[p].y;
            o[3 * p + 2] = result[p].z;
        }
    }
    if (gbuf) std::memcpy(gbuf, sv, sizeof(SVGFBuffer) * (size_t)npx);
    (std::free)(sv);
    (std::free)(result);
    return traversals.load();
}

/* ApplySVGF over width x height pixels, one thread per pixel, __syncthreads
 * = a barrier over all pixels.  result/filtered: npx Vec; prev/cur: npx
 * SVGFBuffer (112 B).  Returns 0, or -1 when the image is too large. */
int ref_svgf(int width, int height, Vec *result, Vec *filtered, void *prev, void *cur, int frame) {
    const int npx = width * height;
    if (npx > 4096 || npx <= 0) return -1;
    image_sizeX_device = width;
    image_sizeY_device = height;
    std::barrier<> bar(npx);
    g_barrier = &bar;
    std::vector<std::thread> th;
    th.reserve(npx);
    for (int p = 0; p < npx; ++p)
        th.emplace_back([=] {
            blockDim.x = 1;
            blockIdx.x = (unsigned)p;
            threadIdx.x = 0;
            ApplySVGF(result, filtered, (SVGFBuffer *)prev, (SVGFBuffer *)cur, 0, 0, frame);
        });
    for (auto &t : th) t.join();
    g_barrier = nullptr;
    return 0;
}

int ref_sizeof_svgfbuffer(void) { return (int)sizeof(SVGFBuffer); }

/* evaluate_Disney_BRDF (outgoing = toward the light, incoming = toward the
 * viewer) and evaluate_Disney_BRDF_pdf for one material and n direction
 * triples (float[3] each).  Material parameters -> alphas and lobe weights as
 * RayTrace.cuh:85-92. */
void ref_disney_eval(const Material *mat, int n, const float *wo, const float *wi,
                     const float *nrm, float *brdf, float *pdf) {
    Material m = *mat;
    float aspect = sqrt(1.0f - 0.9f * m.anisotropic);
    float alpha_sheen = m.roughness * m.roughness;
    float ax = max(0.001f, m.roughness * m.roughness / aspect);
    float ay = max(0.001f, m.roughness * m.roughness * aspect);
    float ac = (1.0f - m.cloearcoatGloss) * 0.1f + m.cloearcoatGloss * 0.001f;
    float w[5] = {0.0f};
    generate_Disney_BRDF_coefficient_array(m, w);
    for (int i = 0; i < n; ++i) {
        Vec o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        Vec in(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        Vec N(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]);
        Vec u, v, ww;
        GenerateONBFromNormal(N, u, v, ww);
        Vec b = evaluate_Disney_BRDF(w, m, o, in, N, u, v, ww, ax, ay, ac);
        brdf[3 * i] = b.x;
        brdf[3 * i + 1] = b.y;
        brdf[3 * i + 2] = b.z;
        pdf[i] = evaluate_Disney_BRDF_pdf(w, in, o, N, u, v, ww, ax, ay, alpha_sheen, ac);
    }
}

/* Camera_SetUpCamera; PixelSize uses the reference's image_sizeY (1080). */
void ref_camera_setup(const float *org, float dist, float rx, float ry, float rz, Camera *out) {
    *out = Camera_SetUpCamera(Vec(org[0], org[1], org[2]), dist, rx, ry, rz);
}

/* Face-light CDF (calculate_Lss) of a scene: out = n floats. */
void ref_light_cdf(const Triangle *tris, int n, const Material *mats, int nm, float *out) {
    HOST_ObjectsData.assign(tris, tris + n);
    HOST_MaterialsData.assign(mats, mats + nm);
    HOST_Light_strength_sum.clear();
    calculate_Lss();
    std::memcpy(out, HOST_Light_strength_sum.data(), sizeof(float) * (size_t)n);
}

/* Environment CDF (calculate_Lss_HDR): out = w*h floats. */
void ref_env_cdf(const float *pixels, int w, int h, int bpp, float *out) {
    g_hdr.pixels = const_cast<float *>(pixels);
    g_hdr.width = w;
    g_hdr.height = h;
    g_hdr.bpp = bpp;
    HOST_HDRData = &g_hdr;
    HOST_Light_strength_sum_HDR.clear();
    calculate_Lss_HDR();
    std::memcpy(out, HOST_Light_strength_sum_HDR.data(), sizeof(float) * (size_t)w * h);
}

/* load_object (IO_load_WavefrontObj.cuh:10-127) + load_Textures run in
 * directory `dir` (the reference reads ./OBJ.obj, its MTL files and textures
 * from the working directory).  Counts out; ref_obj_copy fetches the arrays. */
static std::vector<Material> g_reserved_materials;
int ref_load_obj(const char *dir, int *n_tris, int *n_mats, int *n_tex) {
    if (g_reserved_materials.empty()) g_reserved_materials = HOST_MaterialsData;
    HOST_ObjectsData.clear();
    HOST_MaterialsData = g_reserved_materials;
    HOST_TexturesData.clear();
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1;
    if (chdir(dir) != 0) return -1;
    load_object();
    const int rc = chdir(cwd);
    *n_tris = (int)HOST_ObjectsData.size();
    *n_mats = (int)HOST_MaterialsData.size();
    *n_tex = (int)HOST_TexturesData.size();
    return rc;
}
void ref_obj_copy(Triangle *tris, Material *mats) {
    std::memcpy(tris, HOST_ObjectsData.data(), sizeof(Triangle) * HOST_ObjectsData.size());
    std::memcpy(mats, HOST_MaterialsData.data(), sizeof(Material) * HOST_MaterialsData.size());
}
void ref_obj_texture(int i, int *w, int *h, int *bpp, const float **pixels) {
    *w = HOST_TexturesData[i].width;
    *h = HOST_TexturesData[i].height;
    *bpp = HOST_TexturesData[i].bpp;
    *pixels = HOST_TexturesData[i].pixels;
}

/* tinyobjloader's own parse of one OBJ (the library load_object calls,
 * IO_load_WavefrontObj.cuh:11-28, with its default reader configuration:
 * triangulation on), MTL files looked up in mtl_dir.  Returns 1 when the
 * reader accepts the file, 0 when it rejects it; counts[0..4] = vertices,
 * normals, texcoords, triangles, materials.  ref_tinyobj_copy then gives the
 * attribute arrays, per corner (vertex, texcoord, normal) indices (-1 = none)
 * and per triangle (material, smoothing group, shape). */
static std::vector<float> g_to_v, g_to_vn, g_to_vt;
static std::vector<int> g_to_corner, g_to_face;
int ref_tinyobj_parse(const char *path, const char *mtl_dir, long long *counts) {
    tinyobj::ObjReaderConfig cfg;
    cfg.mtl_search_path = mtl_dir;
    tinyobj::ObjReader reader;
    g_to_v.clear(); g_to_vn.clear(); g_to_vt.clear(); g_to_corner.clear(); g_to_face.clear();
    for (int k = 0; k < 5; ++k) counts[k] = 0;
    if (!reader.ParseFromFile(path, cfg)) return 0;
    const auto &a = reader.GetAttrib();
    g_to_v.assign(a.vertices.begin(), a.vertices.end());
    g_to_vn.assign(a.normals.begin(), a.normals.end());
    g_to_vt.assign(a.texcoords.begin(), a.texcoords.end());
    const auto &shapes = reader.GetShapes();
    for (size_t s = 0; s < shapes.size(); ++s) {
        const auto &m = shapes[s].mesh;
        size_t off = 0;
        for (size_t f = 0; f < m.num_face_vertices.size(); ++f) {
            const size_t fv = m.num_face_vertices[f];
            if (fv == 3) {
                for (size_t v = 0; v < 3; ++v) {
                    const tinyobj::index_t ix = m.indices[off + v];
                    g_to_corner.push_back(ix.vertex_index);
                    g_to_corner.push_back(ix.texcoord_index);
                    g_to_corner.push_back(ix.normal_index);
                }
                g_to_face.push_back(m.material_ids[f]);
                g_to_face.push_back((int)m.smoothing_group_ids[f]);
                g_to_face.push_back((int)s);
            }
            off += fv;
        }
    }
    counts[0] = (long long)g_to_v.size() / 3;
    counts[1] = (long long)g_to_vn.size() / 3;
    counts[2] = (long long)g_to_vt.size() / 2;
    counts[3] = (long long)g_to_face.size() / 3;
    counts[4] = (long long)reader.GetMaterials().size();
    return 1;
}
void ref_tinyobj_copy(float *v, float *vn, float *vt, int *corner, int *face) {
    std::memcpy(v, g_to_v.data(), g_to_v.size() * sizeof(float));
    std::memcpy(vn, g_to_vn.data(), g_to_vn.size() * sizeof(float));
    std::memcpy(vt, g_to_vt.data(), g_to_vt.size() * sizeof(float));
    std::memcpy(corner, g_to_corner.data(), g_to_corner.size() * sizeof(int));
    std::memcpy(face, g_to_face.data(), g_to_face.size() * sizeof(int));
}

/* Writes what the reference's GPU render() needs of a scene to `path`, as
 * render_prepare and main.cu prepare it (construct_BVH, calculate_Lss,
 * Convert_BVHTreeFromHostToDevice): the file read by oracle/ref_gpu.py.
 *   char[8] "KGKREFS1"; int32 n_tris, n_mats, n_nodes, n_faces, n_lss,
 *   exists_nolight; Triangle[n_tris]; Material[n_mats];
 *   BVH_node_Device[n_nodes] with face_list holding the int64 offset of the
 *   node's entries in the face array (-1: none); int32[n_faces];
 *   float[n_lss].  Returns 0, or -1 when the file cannot be written. */
static_assert(sizeof(BVH_node_Device) == 72, "BVH_node_Device");
int ref_export_scene(const Triangle *tris, int n, const Material *mats, int nm, const char *path) {
    load_scene(tris, n, mats, nm);
    HOST_Light_strength_sum.clear();
    HOST_Exists_NoLight = false;
    calculate_Lss();
    std::vector<BVH_node_Device> nodes(g_tree.begin(), g_tree.end());
    std::vector<int> faces;
    for (auto &nd : nodes) {
        long long off = -1;
        if (nd.face_list) {
            off = (long long)faces.size();
            faces.insert(faces.end(), nd.face_list, nd.face_list + nd.face_list_size);
        }
        std::memcpy(&nd.face_list, &off, sizeof off);
    }
    FILE *f = std::fopen(path, "wb");
    if (!f) return -1;
    const int hdr[6] = {n, nm, (int)nodes.size(), (int)faces.size(), (int)HOST_Light_strength_sum.size(),
                        HOST_Exists_NoLight ? 1 : 0};
    bool ok = std::fwrite("KGKREFS1", 1, 8, f) == 8 && std::fwrite(hdr, sizeof hdr, 1, f) == 1;
    ok = ok && std::fwrite(tris, sizeof(Triangle), (size_t)n, f) == (size_t)n;
    ok = ok && std::fwrite(mats, sizeof(Material), (size_t)nm, f) == (size_t)nm;
    ok = ok && std::fwrite(nodes.data(), sizeof(BVH_node_Device), nodes.size(), f) == nodes.size();
    ok = ok && std::fwrite(faces.data(), sizeof(int), faces.size(), f) == faces.size();
    ok = ok && std::fwrite(HOST_Light_strength_sum.data(), sizeof(float), HOST_Light_strength_sum.size(), f) ==
                   HOST_Light_strength_sum.size();
    return (std::fclose(f) == 0 && ok) ? 0 : -1;
}

/* save_png (FileIO/IO_save_png.cuh:34-56) on a full image_sizeX x
 * image_sizeY buffer of Vec (its gamma, clamp and truncation, then
 * stbi_write_png), written as <prefix>000.png and read back with stbi_load:
 * rgba receives the image's bytes (4 per pixel).  Returns 0, or -1 when the
 * file could not be written or read. */
int ref_save_png_bytes(const Vec *image, const char *prefix, unsigned char *rgba) {
    const size_t npx = (size_t)image_sizeX * image_sizeY;
    std::vector<Vec> buf(image, image + npx);   // save_png converts its argument in place
    save_png(buf.data(), 1, prefix);
    const std::string name = std::string(prefix) + "000.png";
    int w = 0, h = 0, comp = 0;
    unsigned char *px = stbi_load(name.c_str(), &w, &h, &comp, 4);
    std::remove(name.c_str());
    if (!px || w != image_sizeX || h != image_sizeY) return -1;
    std::memcpy(rgba, px, npx * 4);
    stbi_image_free(px);
    return 0;
}

int ref_image_size(int *w, int *h) {
    *w = image_sizeX;
    *h = image_sizeY;
    return 0;
}

/* The reference checkout this library was built from (its vendored test
 * models are read from there). */
const char *ref_source_dir(void) { return KGK_REF_DIR; }

/* stbi_loadf of one file (load_image without the +1e-4, and load_HDR). */
const float *ref_load_image(const char *path, int *w, int *h, int *bpp) {
    return stbi_loadf(path, w, h, bpp, 0);
}

} // extern "C"
