// nrc.cu - learned radiance cache: an MLP of hidden width W = 64 or 128
// (64 inputs -> W, 4 x (W -> W), ReLU after each, -> 3 linear outputs, no
// biases) in BF16 on the 5th-generation tensor cores (tcgen05, accumulators
// in tensor memory) with FP32 accumulation.
//
// Inference (k_infer_tc) and the training forward / backward pass
// (k_train_fb_tc) hold the weights once per CTA in shared memory, 128-byte
// swizzled, and carry tiles of 128 samples per warpgroup through the layers;
// the backward pass reads the same weight tiles as MN-major operands.  The
// training pass writes every layer's activations and output gradients (BF16)
// to a scratch by TMA; the weight-gradient GEMM (k_train_dw_tc) reads them
// back by TMA as MN-major operands and accumulates dW in tensor memory.
// Relative-L2 loss with a dynamic loss scale; Adam updates FP32 master
// weights and rewrites the BF16 image.
// No counterpart in the reference.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kgk_device.cuh"
#include "kgk_nrc.h"
#include "kgk_scene.h"

namespace kgk {
namespace nrc {

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&h);
}
// ReLU and BF16 rounding of two values in one conversion (negative values,
// and only those, become 0; lo in the low half).
__device__ __forceinline__ uint32_t pack2_relu(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}
// sin(pi x) and cos(pi x) for the input encoding: x reduced exactly to
// [-1, 1] (x - 2 rint(x / 2)), then the hardware sine and cosine of pi times
// it, whose absolute error (about 1e-6) lies far below the BF16 rounding
// every feature gets before the first layer.
__device__ __forceinline__ void sincospi_feature(float x, float *s, float *c) {
    const float r = x - 2.0f * rintf(0.5f * x);
    __sincosf(r * 3.14159265358979f, s, c);
}

// All 64 input features of a raw query: 3 x 12 sine / cosine features of the
// normalised position (6 octaves), normal and view direction, their sines and
// cosines (12), roughness and albedo, six constant ones (the biases).
__device__ __forceinline__ void encode_row(const float *raw, float (&f)[64]) {
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            float s, co;
            sincospi_feature(raw[ax] * (float)(1 << k), &s, &co);
            f[ax * 12 + 2 * k] = s;
            f[ax * 12 + 2 * k + 1] = co;
        }
    }
#pragma unroll
    for (int j = 0; j < 6; ++j) f[36 + j] = raw[3 + j];  // normal, view
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        float s, co;
        sincospi_feature(raw[3 + j], &s, &co);
        f[42 + 2 * j] = s;
        f[42 + 2 * j + 1] = co;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) f[54 + j] = raw[9 + j];  // roughness, albedo
#pragma unroll
    for (int j = 58; j < 64; ++j) f[j] = 1.0f;
}

// ---------------------------------------------------------------------------
// inference on the 5th-generation tensor cores (tcgen05 + TMEM)
//
// A CTA holds the weights once (BF16, 128-byte-swizzled K-major, in shared
// memory; each layer as K sub-tiles of 64 inputs) for its warpgroups, each
// carrying its own tiles of 128 queries through the network: thread r of a
// warpgroup owns row r.  Per layer a warpgroup writes the BF16 activations
// (128 x W) to its shared-memory tile in the same layout, one elected thread
// issues the tcgen05.mma (M=128, N=W, K=16 each) into the warpgroup's
// 128 x W FP32 accumulator in tensor memory and commits to the warpgroup's
// mbarrier; the threads then read their row back (tcgen05.ld 32x32b) and
// apply the ReLU and the BF16 rounding for the next layer in one conversion.
// The warpgroups synchronise on their own named barriers, so the CUDA-core
// work of one overlaps the MMAs of another.  Width 64: four warpgroups per
// CTA, two CTAs per SM; width 128: two warpgroups, one CTA per SM (shared
// memory).  The output layer uses N=16 (3 live rows of the padded weights).
// Every wait is bounded: on a timeout the CTA raises *err, stops issuing and
// frees its tensor memory.
// ---------------------------------------------------------------------------
namespace tc {

constexpr int kRows = 128;                  // M of every MMA, queries per tile
constexpr uint32_t kSub = kRows * 128;      // activation K sub-tile: 128 rows x 64 BF16
constexpr uint32_t kOutSub = kOutRows * 128;  // output-layer K sub-tile: 16 rows x 64 BF16

template <int W>
struct Tc {
    static constexpr int kGroups = W == 64 ? 4 : 2;  // warpgroups per CTA, one tile each at a time
    static constexpr int kCtasPerSm = W == 64 ? 2 : 1;
    static constexpr uint32_t kKSubs = W / 64;       // K sub-tiles of a W-input layer
    static constexpr uint32_t kWSub = (uint32_t)W * 128;  // weight K sub-tile: W rows x 64 BF16
    // layer l's weights: in(l) / 64 sub-tiles (layer 0: one)
    __host__ __device__ static constexpr uint32_t layer_off(int l) {
        return l == 0 ? 0u : kWSub + (uint32_t)(l - 1) * kKSubs * kWSub;
    }
    static constexpr uint32_t kOutOff = layer_off(kLayers);
    static constexpr uint32_t kAOff = kOutOff + kKSubs * kOutSub;  // activation tiles (1024-aligned)
    static constexpr uint32_t kATile = kKSubs * kSub;
    static constexpr uint32_t kBarOff = kAOff + kGroups * kATile;   // one mbarrier per warpgroup
    static constexpr uint32_t kSlotOff = kBarOff + 8 * kGroups;
    static constexpr uint32_t kSmemBytes = kSlotOff + 8 + 1024;     // + room to align the base to 1024 B
    static constexpr uint32_t kTmemCols = (uint32_t)W * kGroups;    // a W-column accumulator per warpgroup
    // inference: two accumulators per warpgroup when a layer has two K
    // sub-tiles, so the next layer's MMAs on the first sub-tile run while the
    // second is converted
    static constexpr int kAccBufs = kKSubs > 1 ? 2 : 1;
    static constexpr uint32_t kInferTmemCols = kTmemCols * kAccBufs;
    static_assert(kAOff % 1024 == 0, "swizzle atoms need 1024-byte alignment");
    static_assert(kSmemBytes <= 227 * 1024, "shared memory per CTA");
    static_assert(kTmemCols * kCtasPerSm <= 512, "tensor memory per SM");
    static_assert(kInferTmemCols * kCtasPerSm <= 512, "tensor memory per SM (inference)");
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms
// 1024 B apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1u << 16) | ((uint64_t)(1024u >> 4) << 32) |
           ((uint64_t)1u << 46) | ((uint64_t)2u << 61);
}

// Instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 D, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool bar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the barrier phase; false after ~1 s (2^31 SM cycles).
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!bar_try(bar, parity))
        if (clock64() - t0 > (1ll << 31)) return false;
    return true;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Row r of a 128B-swizzled K-major tile: 16-byte chunk c of the row.
__device__ __forceinline__ uint32_t sw_off(int r, int c) { return (uint32_t)r * 128u + ((uint32_t)(c ^ (r & 7)) << 4); }

// The same shared-memory bytes read as an MN-major operand: a 128-byte
// swizzled tile whose rows run along K and whose 64 contiguous elements run
// along M or N (the 128B-swizzle atom is 8 K-rows x 128 B either way).
// lbo = byte distance between 64-element atoms along M / N, sbo = byte
// distance between groups of 8 K-rows.
__device__ __forceinline__ uint64_t sw128_desc_mn(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1u << 46) | ((uint64_t)2u << 61);
}

// Instruction descriptor with B MN-major (bit 16, "transpose B").
__host__ __device__ constexpr uint32_t idesc_bf16_bmn(int M, int N) { return idesc_bf16(M, N) | (1u << 16); }

// TMA store of one 3-D box from shared memory (bulk group of this thread).
__device__ __forceinline__ void tma_store3(const CUtensorMap *map, uint32_t src, int c0, int c1, int c2) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(c0), "r"(c1), "r"(c2), "r"(src)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the bulk stores of this thread have read their shared memory
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// ... and completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace tc

// Named barrier of one warpgroup (ids 1..4; 0 is __syncthreads), and its OR
// reduction.
__device__ __forceinline__ void wg_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
__device__ __forceinline__ bool wg_sync_or(int id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id)
        : "memory");
    return r != 0;
}

template <int W>
__global__ void __launch_bounds__(128 * tc::Tc<W>::kGroups) k_infer_tc(const unsigned short *__restrict__ img,
                                                                       const float *__restrict__ raw,
                                                                       int stride_floats, int n, const int *n_dev,
                                                                       float *out, float4 *rad, int *err) {
    using namespace tc;
    using T = Tc<W>;
    constexpr int kG = T::kGroups, P = Net<W>::kPitch;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t pad = (1024u - (smem_u32(smem_raw) & 1023u)) & 1023u;
    unsigned char *sm = smem_raw + pad;
    const uint32_t s0 = smem_u32(sm);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int g = tid >> 7, r = tid & 127;  // warpgroup, row
    const int wgbar = 1 + g;                // its named barrier
    // weights: BF16 image rows (pitch P) -> swizzled K-major sub-tiles
    constexpr int kChunks = W / 8;  // 16-byte chunks of a W-input row
    for (int i = tid; i < (kLayers * W + kOutRows) * kChunks; i += blockDim.x) {
        const int row = i / kChunks, c = i % kChunks;
        uint32_t dst;
        if (row < kLayers * W) {
            const int l = row / W;
            if (c >= Net<W>::in(l) / 8) continue;
            dst = T::layer_off(l) + (uint32_t)(c >> 3) * T::kWSub + sw_off(row % W, c & 7);
        } else {
            dst = T::kOutOff + (uint32_t)(c >> 3) * kOutSub + sw_off(row - kLayers * W, c & 7);
        }
        *reinterpret_cast<uint4 *>(sm + dst) = *reinterpret_cast<const uint4 *>(img + (size_t)row * P + c * 8);
    }
    const uint32_t bar = s0 + T::kBarOff + 8u * (uint32_t)g;
    if (r == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s0 + T::kSlotOff),
                     "r"(T::kInferTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    constexpr uint32_t kGroupCols = (uint32_t)W * T::kAccBufs;
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(sm + T::kSlotOff) + kGroupCols * (uint32_t)g;
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's 32 TMEM lanes
    const int total = n_dev ? min(*n_dev, n) : n;
    uint32_t phase = 0;
    bool failed = false;
    unsigned char *A = sm + T::kAOff + (uint32_t)g * T::kATile;
    const uint32_t a_addr = s0 + T::kAOff + (uint32_t)g * T::kATile;
    for (int tile = blockIdx.x * kG + g; tile * kRows < total; tile += gridDim.x * kG) {
        const int q = tile * kRows + r;
        const bool live = q < total;
        // input encoding of row r (the first K sub-tile)
        {
            float rw[kRaw];
#pragma unroll
            for (int k = 0; k < kRaw; ++k) rw[k] = live ? raw[(size_t)q * stride_floats + k] : 0.0f;
            float f[64];
            encode_row(rw, f);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                uint4 v;
                v.x = pack2(f[8 * c + 0], f[8 * c + 1]);
                v.y = pack2(f[8 * c + 2], f[8 * c + 3]);
                v.z = pack2(f[8 * c + 4], f[8 * c + 5]);
                v.w = pack2(f[8 * c + 6], f[8 * c + 7]);
                *reinterpret_cast<uint4 *>(A + sw_off(r, c)) = v;
            }
        }
        float y[3] = {0.0f, 0.0f, 0.0f};
        // the MMAs of layer l on K sub-tile h (k-steps 4h .. 4h + 3) into the
        // layer's accumulator; issued by row 0 once the sub-tile is written
        auto issue = [&](int l, int h) {
            const bool last = l == kLayers;
            const uint32_t boff = last ? T::kOutOff : T::layer_off(l);
            const uint32_t bsub = last ? kOutSub : T::kWSub;
            const uint32_t id = last ? idesc_bf16(128, 16) : idesc_bf16(128, W);
            const uint32_t d = tmem + (uint32_t)W * (uint32_t)(l % T::kAccBufs);
            const int nk = Net<W>::in(l) / 16;
            for (int kk = 4 * h; kk < nk && kk < 4 * h + 4; ++kk) {
                const uint32_t j = (uint32_t)kk >> 2, o = 2u * (uint32_t)(kk & 3);  // sub-tile, 32 B steps
                mma_bf16(d, sw128_desc(a_addr + j * kSub) + o, sw128_desc(s0 + boff + j * bsub) + o, id,
                         kk > 0 ? 1u : 0u);
            }
        };
        fence_async_smem();
        fence_before();
        wg_sync(wgbar);
        if (r == 0) {
            fence_after();
            issue(0, 0);
            commit(bar);
        }
        for (int l = 0; l <= kLayers; ++l) {
            const bool ok = bar_wait(bar, phase);
            phase ^= 1u;
            if (wg_sync_or(wgbar, !ok)) {
                failed = true;
                break;
            }
            fence_after();
            const uint32_t acc = trow + (uint32_t)W * (uint32_t)(l % T::kAccBufs);
            if (l == kLayers) {
                float v[16];
                tmem_ld16(acc, v);
                tmem_wait_ld();
                y[0] = v[0];
                y[1] = v[1];
                y[2] = v[2];
                break;
            }
            // tensor-memory loads per wait: four at width 128; one at width
            // 64, whose two CTAs per SM leave 64 registers a thread
            constexpr int kLd = W == 64 ? 1 : 4;
#pragma unroll
            for (int h = 0; h < (int)T::kKSubs; ++h) {  // 64-column K sub-tiles of H_{l+1}
                unsigned char *At = A + (uint32_t)h * kSub;
#pragma unroll
                for (int c0 = 0; c0 < 4; c0 += kLd) {
                    float v[kLd][16];
#pragma unroll
                    for (int c = 0; c < kLd; ++c) tmem_ld16(acc + 64 * h + 16 * (c0 + c), v[c]);
                    tmem_wait_ld();
#pragma unroll
                    for (int c = 0; c < kLd; ++c) {
                        uint4 lo, hi;
                        lo.x = pack2_relu(v[c][0], v[c][1]);
                        lo.y = pack2_relu(v[c][2], v[c][3]);
                        lo.z = pack2_relu(v[c][4], v[c][5]);
                        lo.w = pack2_relu(v[c][6], v[c][7]);
                        hi.x = pack2_relu(v[c][8], v[c][9]);
                        hi.y = pack2_relu(v[c][10], v[c][11]);
                        hi.z = pack2_relu(v[c][12], v[c][13]);
                        hi.w = pack2_relu(v[c][14], v[c][15]);
                        *reinterpret_cast<uint4 *>(At + sw_off(r, 2 * (c0 + c))) = lo;
                        *reinterpret_cast<uint4 *>(At + sw_off(r, 2 * (c0 + c) + 1)) = hi;
                    }
                }
                // sub-tile h of H_{l+1} is written: layer l + 1's MMAs on it
                // start while the next sub-tile is converted
                fence_async_smem();
                fence_before();
                wg_sync(wgbar);
                if (r == 0) {
                    fence_after();
                    issue(l + 1, h);
                    if (h == (int)T::kKSubs - 1) commit(bar);
                }
            }
        }
        if (failed) break;
        if (live) {
            if (out) {
                out[(size_t)q * 3 + 0] = y[0];
                out[(size_t)q * 3 + 1] = y[1];
                out[(size_t)q * 3 + 2] = y[2];
            }
            if (rad) {
                // cache termination: rad[path] += T * max(y, 0)
                const float *rec = raw + (size_t)q * stride_floats;
                const int path = __float_as_int(rec[16]);
                float4 rr = rad[path];
                rr.x += rec[13] * fmaxf(y[0], 0.0f);
                rr.y += rec[14] * fmaxf(y[1], 0.0f);
                rr.z += rec[15] * fmaxf(y[2], 0.0f);
                rad[path] = rr;
            }
        }
    }
    if (failed) {
        // the MMAs of the timed-out phase may still be in flight: wait once
        // more (bounded) before the tensor memory is released
        bar_wait(bar, phase ^ 1u);
        if (r == 0) atomicExch(err, 1);
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem - kGroupCols * (uint32_t)g),
                     "r"(T::kInferTmemCols)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// Training forward and backward on the 5th-generation tensor cores.  The CTA
// layout is k_infer_tc's: the weights once in shared memory (K-major,
// 128-byte swizzle), one 128-sample tile per warpgroup (thread r = row r =
// tensor-memory lane r), a W-column FP32 accumulator per warpgroup.  Per tile:
//   forward   Z_l = H_l W_l^T (A = H_l, B = W_l, both K-major), l = 0..4;
//             H_{l+1} = bf16(relu(Z_l)), the ReLU derivative kept as bits;
//             Y = H_5 W_5^T (N = 16, 3 live outputs);
//   loss      relative L2 against the target, d/dY with the denominator held,
//             times the loss scale: dZ_5 = (dy0, dy1, dy2, 0, ...);
//   backward  dA_{l-1} = dZ_l W_l with the same weight tiles read as an
//             MN-major B operand (K = the layer's outputs along the tile rows,
//             N = its inputs along the swizzled 128-byte rows), and
//             dZ_{l-1} = bf16(dA_{l-1} * relu'(Z_{l-1})), l = 5..1.
// Each H_l and dZ_l tile goes to the global scratch (BF16, W per row, the
// layout k_train_dw_tc reads) by TMA stores of the shared-memory tile the
// layer's MMAs read, issued while they run (dZ_5 and dZ_0, which no MMA
// reads, by the threads); the rows of the last tile past the sample count
// are written too, with dY = 0.  Every mbarrier wait is bounded; a
// timeout sets *err and ends the CTA after a last bounded wait for its MMAs,
// freeing its tensor memory.
// ---------------------------------------------------------------------------
template <int W>
__global__ void __launch_bounds__(128 * tc::Tc<W>::kGroups) k_train_fb_tc(
    const unsigned short *__restrict__ img, const float *__restrict__ raw, int raw_stride,
    const float *__restrict__ target, int tgt_stride, int n, const int *n_dev, const float *scale_p,
    unsigned short *Ds, size_t layer_stride, const __grid_constant__ CUtensorMap tmH,
    const __grid_constant__ CUtensorMap tmD, float *loss_sum, int *err) {
    using namespace tc;
    using T = Tc<W>;
    constexpr int kG = T::kGroups, P = Net<W>::kPitch, kMW = W / 32;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t pad = (1024u - (smem_u32(smem_raw) & 1023u)) & 1023u;
    unsigned char *sm = smem_raw + pad;
    const uint32_t s0 = smem_u32(sm);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int g = tid >> 7, r = tid & 127;
    const int wgbar = 1 + g;
    constexpr int kChunks = W / 8;
    for (int i = tid; i < (kLayers * W + kOutRows) * kChunks; i += blockDim.x) {
        const int row = i / kChunks, c = i % kChunks;
        uint32_t dst;
        if (row < kLayers * W) {
            const int l = row / W;
            if (c >= Net<W>::in(l) / 8) continue;
            dst = T::layer_off(l) + (uint32_t)(c >> 3) * T::kWSub + sw_off(row % W, c & 7);
        } else {
            dst = T::kOutOff + (uint32_t)(c >> 3) * kOutSub + sw_off(row - kLayers * W, c & 7);
        }
        *reinterpret_cast<uint4 *>(sm + dst) = *reinterpret_cast<const uint4 *>(img + (size_t)row * P + c * 8);
    }
    const uint32_t bar = s0 + T::kBarOff + 8u * (uint32_t)g;
    if (r == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s0 + T::kSlotOff),
                     "r"(T::kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(sm + T::kSlotOff) + (uint32_t)W * (uint32_t)g;
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);
    const int total = n_dev ? min(*n_dev, n) : n;
    const int padded = (total + 127) & ~127;  // whole tiles: k_train_dw_tc reads 64-row boxes
    const float S = *scale_p;
    const float inv_n = 1.0f / (3.0f * (float)max(total, 1));
    float lsum = 0.0f;
    uint32_t phase = 0;
    bool failed = false;
    unsigned char *A = sm + T::kAOff + (uint32_t)g * T::kATile;
    const uint32_t a_addr = s0 + T::kAOff + (uint32_t)g * T::kATile;
    // Issues one layer's MMAs into the accumulator (forward: Z = A W^T;
    // backward: dA = A W, the weights read MN-major), then - while they run -
    // the TMA stores of the A tile itself (H_l or dZ_l of the layer, `nsub`
    // sub-tiles of 64 columns, two 64-row boxes each) into the scratch, waits
    // for the MMAs (bounded) and for the stores to have read the tile;
    // false when the wait timed out in any thread of the group.
    auto run_mma = [&](bool backward, int l, const CUtensorMap *map, int nsub, int q0) -> bool {
        fence_async_smem();
        fence_before();
        wg_sync(wgbar);
        if (r == 0) {
            fence_after();
            const bool last = l == kLayers;
            const uint32_t boff = last ? T::kOutOff : T::layer_off(l);
            const uint32_t bsub = last ? kOutSub : T::kWSub;
            if (!backward) {
                const int nk = Net<W>::in(l) / 16;
                const uint32_t id = last ? idesc_bf16(128, 16) : idesc_bf16(128, W);
                for (int kk = 0; kk < nk; ++kk) {
                    const uint32_t j = (uint32_t)kk >> 2, o = 2u * (uint32_t)(kk & 3);
                    mma_bf16(tmem, sw128_desc(a_addr + j * kSub) + o, sw128_desc(s0 + boff + j * bsub) + o, id,
                             kk > 0 ? 1u : 0u);
                }
            } else {
                // K = layer l's outputs (16 rows of the output layer, else W),
                // N = its W inputs in W / 64 atoms, the sub-tiles bsub apart
                const int nk = last ? 1 : W / 16;
                const uint32_t id = idesc_bf16_bmn(128, W);
                for (int kk = 0; kk < nk; ++kk) {
                    const uint32_t j = (uint32_t)kk >> 2, o = 2u * (uint32_t)(kk & 3);
                    mma_bf16(tmem, sw128_desc(a_addr + j * kSub) + o,
                             sw128_desc_mn(s0 + boff + (uint32_t)kk * 2048u, bsub, 1024u), id, kk > 0 ? 1u : 0u);
                }
            }
            commit(bar);
            if (map) {
                for (int jj = 0; jj < nsub; ++jj)
                    for (int h = 0; h < 2; ++h)
                        tma_store3(map, a_addr + (uint32_t)jj * kSub + (uint32_t)h * 8192u, 64 * jj, q0 + 64 * h, l);
                bulk_commit();
            }
        }
        const bool ok = bar_wait(bar, phase);
        phase ^= 1u;
        if (r == 0 && map) bulk_wait_read();  // the tile may be overwritten after the barrier below
        if (wg_sync_or(wgbar, !ok)) return false;
        fence_after();
        return true;
    };
    for (int tile = blockIdx.x * kG + g; tile * kRows < padded; tile += gridDim.x * kG) {
        const int q0 = tile * kRows, q = q0 + r;
        const bool live = q < total;
        unsigned short *drow = Ds + (size_t)q * W;
        {
            float rw[kRaw];
#pragma unroll
            for (int k = 0; k < kRaw; ++k) rw[k] = live ? raw[(size_t)q * raw_stride + k] : 0.0f;
            float f[64];
            encode_row(rw, f);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                uint4 v;
                v.x = pack2(f[8 * c + 0], f[8 * c + 1]);
                v.y = pack2(f[8 * c + 2], f[8 * c + 3]);
                v.z = pack2(f[8 * c + 4], f[8 * c + 5]);
                v.w = pack2(f[8 * c + 6], f[8 * c + 7]);
                *reinterpret_cast<uint4 *>(A + sw_off(r, c)) = v;
            }
        }
        uint32_t msk[kLayers][kMW];
        float y[3] = {0.0f, 0.0f, 0.0f};
        for (int l = 0; l <= kLayers; ++l) {
            // H_l goes to the scratch while its layer's MMAs run
            if (!run_mma(false, l, &tmH, l == 0 ? 1 : W / 64, q0)) {
                failed = true;
                break;
            }
            if (l < kLayers) {
#pragma unroll
                for (int hb = 0; hb < W / 64; ++hb) {  // 64 columns per tensor-memory wait
                    float v[4][16];
#pragma unroll
                    for (int c = 0; c < 4; ++c) tmem_ld16(trow + 64 * hb + 16 * c, v[c]);
                    tmem_wait_ld();
#pragma unroll
                    for (int c = 0; c < 4; ++c) {
                        const int cb = 4 * hb + c;
                        uint32_t bits = 0;
#pragma unroll
                        for (int i = 0; i < 16; ++i) bits |= (v[c][i] > 0.0f ? 1u : 0u) << i;
                        if (cb & 1) msk[l][cb >> 1] |= bits << 16;
                        else msk[l][cb >> 1] = bits;
                        uint4 lo, hi;
                        lo.x = pack2_relu(v[c][0], v[c][1]);
                        lo.y = pack2_relu(v[c][2], v[c][3]);
                        lo.z = pack2_relu(v[c][4], v[c][5]);
                        lo.w = pack2_relu(v[c][6], v[c][7]);
                        hi.x = pack2_relu(v[c][8], v[c][9]);
                        hi.y = pack2_relu(v[c][10], v[c][11]);
                        hi.z = pack2_relu(v[c][12], v[c][13]);
                        hi.w = pack2_relu(v[c][14], v[c][15]);
                        unsigned char *At = A + (uint32_t)hb * kSub;
                        *reinterpret_cast<uint4 *>(At + sw_off(r, (2 * cb) & 7)) = lo;
                        *reinterpret_cast<uint4 *>(At + sw_off(r, (2 * cb + 1) & 7)) = hi;
                    }
                }
            } else {
                float v[16];
                tmem_ld16(trow, v);
                tmem_wait_ld();
                y[0] = v[0];
                y[1] = v[1];
                y[2] = v[2];
            }
        }
        if (failed) break;
        // relative L2: d/dy (y - t)^2 / (y^2 + eps), denominator held constant
        float dy[3] = {0.0f, 0.0f, 0.0f};
        if (live) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float tt = target[(size_t)q * tgt_stride + c];
                const float den = y[c] * y[c] + kEpsRel;
                const float d = y[c] - tt;
                lsum += d * d / den;
                dy[c] = 2.0f * d / den * inv_n * S;
            }
        }
        {
            // dZ_5: 16 columns (chunks 0 and 1 of the first sub-tile), 3 live;
            // its scratch row by the thread (columns 0..7; 8.. stay zero)
            uint4 lo;
            lo.x = pack2(dy[0], dy[1]);
            lo.y = pack2(dy[2], 0.0f);
            lo.z = 0u;
            lo.w = 0u;
            *reinterpret_cast<uint4 *>(A + sw_off(r, 0)) = lo;
            *reinterpret_cast<uint4 *>(A + sw_off(r, 1)) = make_uint4(0u, 0u, 0u, 0u);
            *reinterpret_cast<uint4 *>(drow + (size_t)kLayers * layer_stride) = lo;
        }
        for (int l = kLayers; l >= 1; --l) {
            // dA_{l-1} = dZ_l W_l; dZ_l (l < kLayers) goes to the scratch meanwhile
            if (!run_mma(true, l, l < kLayers ? &tmD : nullptr, W / 64, q0)) {
                failed = true;
                break;
            }
            // dZ_{l-1} = dA_{l-1} * relu'(Z_{l-1}): into the tile for the next
            // backward MMA, or (dZ_0) straight to the scratch
            unsigned short *dout = drow + (size_t)(l - 1) * layer_stride;
#pragma unroll
            for (int hb = 0; hb < W / 64; ++hb) {
                float v[4][16];
#pragma unroll
                for (int c = 0; c < 4; ++c) tmem_ld16(trow + 64 * hb + 16 * c, v[c]);
                tmem_wait_ld();
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int cb = 4 * hb + c;
                    const uint32_t bits = msk[l - 1][cb >> 1] >> (16 * (cb & 1));
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (!((bits >> i) & 1u)) v[c][i] = 0.0f;
                    uint4 lo, hi;
                    lo.x = pack2(v[c][0], v[c][1]);
                    lo.y = pack2(v[c][2], v[c][3]);
                    lo.z = pack2(v[c][4], v[c][5]);
                    lo.w = pack2(v[c][6], v[c][7]);
                    hi.x = pack2(v[c][8], v[c][9]);
                    hi.y = pack2(v[c][10], v[c][11]);
                    hi.z = pack2(v[c][12], v[c][13]);
                    hi.w = pack2(v[c][14], v[c][15]);
                    if (l > 1) {
                        unsigned char *At = A + (uint32_t)hb * kSub;
                        *reinterpret_cast<uint4 *>(At + sw_off(r, (2 * cb) & 7)) = lo;
                        *reinterpret_cast<uint4 *>(At + sw_off(r, (2 * cb + 1) & 7)) = hi;
                    } else {
                        *reinterpret_cast<uint4 *>(dout + 16 * cb) = lo;
                        *reinterpret_cast<uint4 *>(dout + 16 * cb + 8) = hi;
                    }
                }
            }
        }
        if (failed) break;
    }
    if (failed) {
        bar_wait(bar, phase ^ 1u);
        if (r == 0) atomicExch(err, 1);
    }
    if (r == 0) bulk_wait_all();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(~0u, lsum, o);
    if ((tid & 31) == 0 && loss_sum) atomicAdd(loss_sum, lsum * inv_n);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem - (uint32_t)W * (uint32_t)g),
                     "r"(T::kTmemCols)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
// Weight gradients on the tensor cores: dW_l = dZ_l^T H_l over the batch, as
// D[M = layer outputs x N = layer inputs] += A[M x K] B[K x N], K = samples.
// Both operands come straight from the row-major scratch (one sample's W
// outputs or inputs contiguous per row): read along K they are MN-major
// tiles.  TMA loads boxes of 64 samples x 64 columns with the 128-byte
// swizzle into a ring of stages; one thread feeds the ring, one issues the
// MMAs (K = 16 per instruction, four per stage) and frees each stage with a
// commit; the FP32 accumulator (M = 128 lanes, N <= 128 columns) stays in
// tensor memory for the CTA's whole chunk of samples and is added to the
// global gradient once at the end.  A layer with fewer than 128 outputs
// (64 at width 64, 3 for the output layer) reads its 64-column box twice
// (LBO 0) and keeps only its rows.  Every wait is bounded (~1 s); a timeout
// sets *err, and the CTA waits (bounded) for its loads and MMAs in flight
// before it frees its tensor memory.
// ---------------------------------------------------------------------------
namespace dwt {
constexpr uint32_t kBox = 64u * 128u;  // 64 rows x 64 BF16, one swizzle-atom column
template <int W>
struct Cfg {
    static constexpr int kBoxes = W / 64;  // boxes per operand per stage
    static constexpr int kStages = W == 64 ? 6 : 3;  // 96 KB of stages either way: two CTAs per SM
    static constexpr uint32_t kStage = 2u * kBoxes * kBox;
    static constexpr uint32_t kBarOff = kStages * kStage;  // full[kStages], empty[kStages], done
    static constexpr uint32_t kSlotOff = kBarOff + 8u * (2 * kStages + 1);
    static constexpr uint32_t kSmem = kSlotOff + 16 + 1024;
    static constexpr uint32_t kCols = 128;
};

__device__ __forceinline__ void arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load3(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2,
                                          uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}
}  // namespace dwt

template <int W>
__global__ void __launch_bounds__(128) k_train_dw_tc(const __grid_constant__ CUtensorMap tmH,
                                                     const __grid_constant__ CUtensorMap tmD, int n,
                                                     const int *n_dev, int chunk, float *dW_glob, int *err) {
    using namespace tc;
    using C = dwt::Cfg<W>;
    constexpr int S = C::kStages;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    const uint32_t pad = (1024u - (smem_u32(smem_raw) & 1023u)) & 1023u;
    unsigned char *sm = smem_raw + pad;
    const uint32_t s0a = smem_u32(sm);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int l = blockIdx.y;
    const int total = n_dev ? min(*n_dev, n) : n;
    const int padded = (total + 127) & ~127;  // k_train_fb_tc writes whole 128-row tiles
    const int r0 = blockIdx.x * chunk, r1 = min(r0 + chunk, padded);
    if (r0 >= r1) return;
    const int nst = (r1 - r0) / 64;
    const bool out_layer = l == kLayers;
    const int in = Net<W>::in(l), outs = out_layer ? 3 : W;
    const int ma = out_layer ? 1 : W / 64, nb = in / 64;
    const uint32_t tx = (uint32_t)(ma + nb) * dwt::kBox;
    const uint32_t fullb = s0a + C::kBarOff, emptyb = fullb + 8u * S, doneb = fullb + 16u * S;
    __shared__ int failed_sh;
    if (tid == 0) {
        failed_sh = 0;
        for (int i = 0; i < 2 * S + 1; ++i)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(fullb + 8u * i) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s0a + C::kSlotOff),
                     "r"(C::kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(sm + C::kSlotOff);
    if (tid == 0) {
        // producer: stage i of the chunk into slot i % S
        int issued = 0;
        for (int i = 0; i < nst; ++i) {
            const int s = i % S;
            if (i >= S && !bar_wait(emptyb + 8u * s, (uint32_t)((i / S) - 1) & 1u)) {
                atomicExch(&failed_sh, 1);
                break;
            }
            if (*reinterpret_cast<volatile int *>(&failed_sh)) break;
            const uint32_t st = s0a + (uint32_t)s * C::kStage;
            dwt::arrive_expect_tx(fullb + 8u * s, tx);
            const int row = r0 + 64 * i;
            for (int b = 0; b < ma; ++b) dwt::tma_load3(st + (uint32_t)b * dwt::kBox, &tmD, 64 * b, row, l, fullb + 8u * s);
            for (int b = 0; b < nb; ++b)
                dwt::tma_load3(st + (uint32_t)(C::kBoxes + b) * dwt::kBox, &tmH, 64 * b, row, l, fullb + 8u * s);
            issued = i + 1;
        }
        // every load issued has landed before the CTA's shared memory is released
        for (int i = max(0, issued - S); i < issued; ++i) bar_wait(fullb + 8u * (i % S), (uint32_t)(i / S) & 1u);
    } else if (tid == 32) {
        // MMA issuer: A = dZ (M = outputs, MN-major), B = H (N = inputs, MN-major)
        const uint32_t idesc = idesc_bf16(128, 64 * nb) | (1u << 15) | (1u << 16);
        const uint32_t lboA = ma == 2 ? dwt::kBox : 0u, lboB = nb == 2 ? dwt::kBox : 0u;
        for (int i = 0; i < nst; ++i) {
            const int s = i % S;
            if (!bar_wait(fullb + 8u * s, (uint32_t)(i / S) & 1u)) {
                atomicExch(&failed_sh, 1);
                break;
            }
            fence_after();
            const uint32_t st = s0a + (uint32_t)s * C::kStage;
            const uint32_t bs = st + (uint32_t)C::kBoxes * dwt::kBox;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
                mma_bf16(tmem, sw128_desc_mn(st + (uint32_t)kk * 2048u, lboA, 1024u),
                         sw128_desc_mn(bs + (uint32_t)kk * 2048u, lboB, 1024u), idesc, (i > 0 || kk > 0) ? 1u : 0u);
            commit(emptyb + 8u * s);
        }
        commit(doneb);  // completes once every MMA issued above has
    }
    __syncwarp();
    const bool done_ok = bar_wait(doneb, 0u);
    const bool ok = !__syncthreads_or(!done_ok || failed_sh);  // uniform over the CTA
    fence_after();
    // epilogue: warp w holds rows 32 w .. 32 w + 31 (tensor-memory lanes)
    const int m = 32 * warp + lane;
    float *dW = dW_glob + Net<W>::woff(l);
    if (ok && 32 * warp < outs) {
        for (int c = 0; c < 64 * nb; c += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)c, v);
            tmem_wait_ld();
            if (m < outs) {
#pragma unroll
                for (int k = 0; k < 16; ++k) atomicAdd(dW + (size_t)m * in + c + k, v[k]);
            }
        }
    }
    if (!ok && tid == 0) atomicExch(err, 1);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(C::kCols) : "memory");
    }
}

// Master weights -> padded BF16 image: row r of layer l at (l W + r) P, the
// output layer's 16 rows (3 live) after the hidden layers.
template <int W>
__global__ void k_make_image(const float *w, unsigned short *img) {
    constexpr int P = Net<W>::kPitch;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Net<W>::kImg; i += gridDim.x * blockDim.x) {
        const int row = i / P, c = i % P;
        float v = 0.0f;
        if (row < kLayers * W) {
            const int l = row / W, r = row % W, in = Net<W>::in(l);
            if (c < in) v = w[Net<W>::woff(l) + r * in + c];
        } else {
            const int r = row - kLayers * W;
            if (r < 3 && c < W) v = w[Net<W>::woff(kLayers) + r * W + c];
        }
        __nv_bfloat16 b = __float2bfloat16_rn(v);
        img[i] = *reinterpret_cast<unsigned short *>(&b);
    }
}

// One Adam step with the BF16 image kept in step: every block first checks
// that all gradients are finite (n <= 74,112 floats, read from L2), block 0
// records the verdict for k_scale_update, and if it is clean each updated
// master weight is written to the image too (the image's padding never
// changes).
template <int W>
__global__ void k_adam_image(float *w, float *m, float *v, const float *g, const float *scale_p, float lr, float b1,
                             float b2, float eps, float bc1, float bc2, unsigned short *img, int *bad_out) {
    constexpr int n = Net<W>::kParams, P = Net<W>::kPitch;
    int local = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (!isfinite(g[i])) local = 1;
    const int bad = __syncthreads_or(local);
    if (blockIdx.x == 0 && threadIdx.x == 0) *bad_out = bad;
    if (bad) return;
    const float inv_s = 1.0f / *scale_p;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i] * inv_s;
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
        w[i] = wi;
        // its place in the image: layer l, row r, column c
        int row, c;
        if (i < Net<W>::woff(1)) {
            row = i / kIn;
            c = i % kIn;
        } else if (i < Net<W>::woff(kLayers)) {
            const int k = i - Net<W>::woff(1);
            row = W + k / W;  // layers 1..4 follow layer 0's W rows
            c = k % W;
        } else {
            const int k = i - Net<W>::woff(kLayers);
            row = kLayers * W + k / W;
            c = k % W;
        }
        __nv_bfloat16 bw = __float2bfloat16_rn(wi);
        img[row * P + c] = *reinterpret_cast<unsigned short *>(&bw);
    }
}

// Dynamic loss scaling: halve on a non-finite gradient, double after
// kScaleGrowth clean steps.
__global__ void k_scale_update(float *scale, int *good, const int *bad) {
    if (*bad) {
        *scale = fmaxf(*scale * 0.5f, 1.0f);
        *good = 0;
    } else if (++*good >= kScaleGrowth) {
        *scale = fminf(*scale * 2.0f, 65536.0f);
        *good = 0;
    }
}

__global__ void k_unscale(const float *g, int n, const float *scale_p, float *out) {
    const float inv = 1.0f / *scale_p;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = g[i] * inv;
}

}  // namespace nrc

// ---------------------------------------------------------------------------
// state
// ---------------------------------------------------------------------------
using namespace nrc;

namespace {
// BF16 image of the master weights, on stream st
void make_image(NrcState &N, cudaStream_t st) {
    if (N.cfg.width == 128) k_make_image<128><<<64, 256, 0, st>>>(N.w, N.img);
    else k_make_image<64><<<64, 256, 0, st>>>(N.w, N.img);
}

template <int W>
void launch_infer(NrcState &N, const float *raw, int stride, int n, const int *n_dev, float *out, float4 *rad,
                  cudaStream_t st) {
    using T = tc::Tc<W>;
    k_infer_tc<W><<<N.sms * T::kCtasPerSm, 128 * T::kGroups, T::kSmemBytes, st>>>(N.img, raw, stride, n, n_dev, out,
                                                                                  rad, N.ints + 2);
}

// cuTensorMapEncodeTiled, through the runtime's driver entry point.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// A training scratch (BF16 rows of W, kLayers + 1 layers of `cap` rows) as a
// 3-D TMA tensor (columns, rows, layer) read in 64 x 64 boxes, 128-byte swizzle.
kgk_status scratch_map(CUtensorMap *m, unsigned short *base, int W, int cap) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return fail(KGK_ERR_CUDA, "radiance cache: cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[3] = {(cuuint64_t)W, (cuuint64_t)cap, (cuuint64_t)(kLayers + 1)};
    const cuuint64_t strides[2] = {(cuuint64_t)W * 2, (cuuint64_t)cap * W * 2};
    const cuuint32_t box[3] = {64, 64, 1}, es[3] = {1, 1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS)
        return fail(KGK_ERR_CUDA, "radiance cache: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return KGK_OK;
}

template <int W>
kgk_status launch_grad(NrcState &N, const float *raw, int raw_stride, const float *tgt, int tgt_stride, int n,
                       const int *n_dev, int rows, cudaStream_t st) {
    const size_t ls = (size_t)N.tr_cap * W;
    using T = tc::Tc<W>;
    CUtensorMap mh, md;
    KGK_TRY(scratch_map(&mh, N.trH, W, N.tr_cap));
    KGK_TRY(scratch_map(&md, N.trD, W, N.tr_cap));
    // as many CTAs as the batch's 128-row tiles need (one per warpgroup), at most the resident count
    const int fb_ctas = std::max(1, std::min(N.sms * T::kCtasPerSm, ((n + 127) / 128 + T::kGroups - 1) / T::kGroups));
    k_train_fb_tc<W><<<fb_ctas, 128 * T::kGroups, T::kSmemBytes, st>>>(
        N.img, raw, raw_stride, tgt, tgt_stride, n, n_dev, N.scal, N.trD, ls, mh, md, N.scal + 1, N.ints + 2);
    // split K: chunks of whole 64-row boxes, about two CTAs per SM over the six layers
    const int want = std::max(1, 2 * N.sms / (kLayers + 1));
    int chunk = std::max(1024, (rows + want - 1) / want);
    chunk = (chunk + 63) & ~63;
    const dim3 gdw((unsigned)((rows + chunk - 1) / chunk), kLayers + 1);
    k_train_dw_tc<W><<<gdw, 128, dwt::Cfg<W>::kSmem, st>>>(mh, md, n, n_dev, chunk, N.g, N.ints + 2);
    return KGK_OK;
}
}  // namespace

kgk_status nrc_init(NrcState &N, const kgk_nrc_config *cfg, int device) {
    nrc_free(N);
    if (cfg) N.cfg = *cfg;
    if (N.cfg.width == 0) N.cfg.width = 64;
    if (N.cfg.hidden_layers == 0) N.cfg.hidden_layers = kLayers;
    if (!width_ok(N.cfg.width) || N.cfg.hidden_layers != kLayers)
        return fail(KGK_ERR_UNSUPPORTED, "radiance cache: this build has 5 hidden layers of width 64 or 128");
    const int W = N.cfg.width;
    N.params = params_of(W);
    if (N.cfg.learning_rate <= 0.0f) N.cfg.learning_rate = 1e-2f;
    if (N.cfg.train_paths <= 0) N.cfg.train_paths = 65536;
    if (N.cfg.train_suffix_max <= 0) N.cfg.train_suffix_max = 4;
    if (N.cfg.train_steps <= 0) N.cfg.train_steps = 4;
    if (N.cfg.spread_c <= 0.0f) N.cfg.spread_c = 0.01f;
    KGK_TRY(dalloc(&N.w, (size_t)N.params, "cache weights"));
    KGK_TRY(dalloc(&N.m, (size_t)N.params, "cache Adam state"));
    KGK_TRY(dalloc(&N.v, (size_t)N.params, "cache Adam state"));
    KGK_TRY(dalloc(&N.g, (size_t)N.params, "cache gradient"));
    KGK_TRY(dalloc(&N.img, (size_t)img_elems_of(W), "cache BF16 weights"));
    KGK_TRY(dalloc(&N.scal, 4, "cache scalars"));
    KGK_TRY(dalloc(&N.ints, 4, "cache scalars"));
    // He-uniform initialisation (bound sqrt(6 / inputs of the layer)) from a
    // seeded stream
    std::vector<float> h(N.params);
    unsigned long long s = N.cfg.seed ? N.cfg.seed : 0x1234567ull;
    auto nxt = [&]() {
        s ^= s << 13; s ^= s >> 7; s ^= s << 17;
        return (double)(s >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int i = 0; i < N.params; ++i) {
        const int fan_in = i < W * kIn ? kIn : W;
        h[i] = (float)((2.0 * nxt() - 1.0) * std::sqrt(6.0 / fan_in));
    }
    KGK_CUDA(cudaMemcpy(N.w, h.data(), N.params * sizeof(float), cudaMemcpyHostToDevice));
    KGK_CUDA(cudaMemset(N.m, 0, N.params * sizeof(float)));
    KGK_CUDA(cudaMemset(N.v, 0, N.params * sizeof(float)));
    const float sc[4] = {kInitScale, 0.0f, 0.0f, 0.0f};
    KGK_CUDA(cudaMemcpy(N.scal, sc, sizeof sc, cudaMemcpyHostToDevice));
    KGK_CUDA(cudaMemset(N.ints, 0, 4 * sizeof(int)));
    make_image(N, 0);
    KGK_CUDA(cudaGetLastError());
    KGK_CUDA(cudaDeviceSynchronize());
    KGK_CUDA(cudaFuncSetAttribute(k_train_dw_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)dwt::Cfg<64>::kSmem));
    KGK_CUDA(cudaFuncSetAttribute(k_train_dw_tc<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)dwt::Cfg<128>::kSmem));
    KGK_CUDA(cudaFuncSetAttribute(k_train_fb_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)tc::Tc<64>::kSmemBytes));
    KGK_CUDA(cudaFuncSetAttribute(k_train_fb_tc<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)tc::Tc<128>::kSmemBytes));
    KGK_CUDA(cudaFuncSetAttribute(k_infer_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)tc::Tc<64>::kSmemBytes));
    KGK_CUDA(cudaFuncSetAttribute(k_infer_tc<128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)tc::Tc<128>::kSmemBytes));
    cudaDeviceProp p;
    KGK_CUDA(cudaGetDeviceProperties(&p, device));
    N.sms = p.multiProcessorCount;
    N.step = 0;
    N.ready = true;
    return KGK_OK;
}

void nrc_free(NrcState &N) {
    void *ptrs[] = {N.w, N.m, N.v, N.g, N.img, N.scal, N.ints, N.trH, N.trD};
    for (void *p : ptrs) dfree(p);
    N.w = N.m = N.v = N.g = N.scal = nullptr;
    N.img = N.trH = N.trD = nullptr;
    N.tr_cap = 0;
    N.ints = nullptr;
    N.ready = false;
}

kgk_status nrc_check_error(NrcState &N) {
    int e = 0;
    KGK_CUDA(cudaMemcpy(&e, N.ints + 2, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        KGK_CUDA(cudaMemset(N.ints + 2, 0, sizeof(int)));
        return fail(KGK_ERR_DEVICE_CHECK, "radiance cache: a tensor-core wait timed out (inference abandoned)");
    }
    return KGK_OK;
}

kgk_status nrc_infer_dev(NrcState &N, const float *raw, int stride, int n, const int *n_dev, float *out, float4 *rad,
                         cudaStream_t st) {
    // width 64: two ~107 KB CTAs of four warpgroups per SM (2 x 256 TMEM columns of 512);
    // width 128: one ~213 KB CTA of two warpgroups per SM
    if (N.cfg.width == 128) launch_infer<128>(N, raw, stride, n, n_dev, out, rad, st);
    else launch_infer<64>(N, raw, stride, n, n_dev, out, rad, st);
    KGK_CUDA(cudaGetLastError());
    return KGK_OK;
}

kgk_status nrc_grad_dev(NrcState &N, const float *raw, int raw_stride, const float *tgt, int tgt_stride, int n,
                        const int *n_dev, cudaStream_t st) {
    const int rows = (n + 127) & ~127;  // whole 128-row tiles
    if (N.tr_cap < rows) {
        // per-sample activations and output gradients of every layer (BF16 rows of W)
        dfree(N.trH);
        dfree(N.trD);
        N.trH = N.trD = nullptr;
        N.tr_cap = 0;
        const size_t cnt = (size_t)(kLayers + 1) * rows * N.cfg.width;
        KGK_TRY(dalloc(&N.trH, cnt, "cache training scratch"));
        KGK_TRY(dalloc(&N.trD, cnt, "cache training scratch"));
        KGK_CUDA(cudaMemset(N.trH, 0, cnt * sizeof(unsigned short)));
        KGK_CUDA(cudaMemset(N.trD, 0, cnt * sizeof(unsigned short)));  // output-layer columns >= 8 stay 0
        N.tr_cap = rows;
    }
    KGK_CUDA(cudaMemsetAsync(N.g, 0, N.params * sizeof(float), st));
    KGK_CUDA(cudaMemsetAsync(N.scal + 1, 0, sizeof(float), st));  // loss
    if (N.cfg.width == 128) KGK_TRY(launch_grad<128>(N, raw, raw_stride, tgt, tgt_stride, n, n_dev, rows, st));
    else KGK_TRY(launch_grad<64>(N, raw, raw_stride, tgt, tgt_stride, n, n_dev, rows, st));
    KGK_CUDA(cudaGetLastError());
    return KGK_OK;
}

kgk_status nrc_step_dev(NrcState &N, cudaStream_t st) {
    ++N.step;
    const float b1 = 0.9f, b2 = 0.99f;
    const float bc1 = 1.0f - std::pow(b1, (float)N.step), bc2 = 1.0f - std::pow(b2, (float)N.step);
    // Adam and the image in one launch (the finite check in every block),
    // then the loss scale from block 0's verdict in N.ints[0]
    if (N.cfg.width == 128)
        k_adam_image<128><<<64, 256, 0, st>>>(N.w, N.m, N.v, N.g, N.scal, N.cfg.learning_rate, b1, b2, 1e-10f, bc1,
                                              bc2, N.img, N.ints);
    else
        k_adam_image<64><<<64, 256, 0, st>>>(N.w, N.m, N.v, N.g, N.scal, N.cfg.learning_rate, b1, b2, 1e-10f, bc1,
                                             bc2, N.img, N.ints);
    k_scale_update<<<1, 1, 0, st>>>(N.scal, N.ints + 1, N.ints);
    KGK_CUDA(cudaGetLastError());
    return KGK_OK;
}

NrcState *nrc_state(kgk_scene *s) {
    if (!s->nrc) s->nrc = new NrcState();
    return s->nrc;
}

void nrc_state_free(kgk_scene *s) {
    if (!s->nrc) return;
    nrc_free(*s->nrc);
    delete s->nrc;
    s->nrc = nullptr;
}

}  // namespace kgk

using namespace kgk;

namespace {

kgk_status stage_in(kgk_scene *s, const void *src, size_t bytes, void **dst, std::vector<void *> &owned) {
    if (is_device_ptr(src)) {
        *dst = const_cast<void *>(src);
        return KGK_OK;
    }
    KGK_TRY(dmalloc(dst, bytes, "cache staging"));
    owned.push_back(*dst);
    KGK_CUDA(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, s->stream));
    return KGK_OK;
}

struct Owned {
    std::vector<void *> v;
    ~Owned() {
        for (void *p : v) dfree(p);
    }
};

kgk_status need(kgk_scene *s) {
    if (!s) return fail(KGK_ERR_INVALID_ARGUMENT, "radiance cache: scene == NULL");
    if (!s->nrc || !s->nrc->ready) return fail(KGK_ERR_INVALID_ARGUMENT, "radiance cache: call kgk_nrc_init first");
    KGK_CUDA(cudaSetDevice(s->device));
    return KGK_OK;
}

}  // namespace

extern "C" {

kgk_status kgk_nrc_init(kgk_scene *s, const kgk_nrc_config *cfg) {
    if (!s) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_nrc_init: scene == NULL");
    KGK_CUDA(cudaSetDevice(s->device));
    return nrc_init(*nrc_state(s), cfg, s->device);
}

kgk_status kgk_nrc_set_weights(kgk_scene *s, const float *w, size_t n) {
    KGK_TRY(need(s));
    NrcState &N = *s->nrc;
    if (!w || n != (size_t)N.params)
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_nrc_set_weights: expected " + std::to_string(N.params) + " floats");
    KGK_CUDA(cudaMemcpy(N.w, w, n * sizeof(float), is_device_ptr(w) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    make_image(N, s->stream);
    KGK_CUDA(cudaGetLastError());
    KGK_CUDA(cudaStreamSynchronize(s->stream));
    return KGK_OK;
}

kgk_status kgk_nrc_get_weights(kgk_scene *s, float *w, size_t n) {
    KGK_TRY(need(s));
    if (!w || n != (size_t)s->nrc->params)
        return fail(KGK_ERR_INVALID_ARGUMENT,
                    "kgk_nrc_get_weights: expected " + std::to_string(s->nrc->params) + " floats");
    KGK_CUDA(cudaStreamSynchronize(s->stream));
    KGK_CUDA(cudaMemcpy(w, s->nrc->w, n * sizeof(float), is_device_ptr(w) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost));
    return KGK_OK;
}

kgk_status kgk_nrc_infer(kgk_scene *s, const float *raw, size_t n, float *out) {
    KGK_TRY(need(s));
    if (n == 0) return KGK_OK;
    if (!raw || !out || n > (1u << 30)) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_nrc_infer: bad arguments");
    Owned o;
    void *draw, *dout;
    KGK_TRY(stage_in(s, raw, n * kRaw * sizeof(float), &draw, o.v));
    const bool od = is_device_ptr(out);
    if (od) dout = out;
    else {
        KGK_TRY(dmalloc(&dout, n * 3 * sizeof(float), "cache staging"));
        o.v.push_back(dout);
    }
    KGK_TRY(nrc_infer_dev(*s->nrc, (const float *)draw, kRaw, (int)n, nullptr, (float *)dout, nullptr, s->stream));
    if (!od) KGK_CUDA(cudaMemcpyAsync(out, dout, n * 3 * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    KGK_CUDA(cudaStreamSynchronize(s->stream));
    return nrc_check_error(*s->nrc);
}

kgk_status kgk_nrc_gradients(kgk_scene *s, const float *raw, const float *target, size_t n, float *grad, float *loss) {
    KGK_TRY(need(s));
    if (!raw || !target || !grad || n == 0 || n > (1u << 30))
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_nrc_gradients: bad arguments");
    if (is_device_ptr(grad) || (loss && is_device_ptr(loss)))
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_nrc_gradients: grad and loss must be host memory");
    Owned o;
    void *draw, *dt;
    KGK_TRY(stage_in(s, raw, n * kRaw * sizeof(float), &draw, o.v));
    KGK_TRY(stage_in(s, target, n * 3 * sizeof(float), &dt, o.v));
    NrcState &N = *s->nrc;
    KGK_TRY(nrc_grad_dev(N, (const float *)draw, kRaw, (const float *)dt, 3, (int)n, nullptr, s->stream));
    void *dg;
    KGK_TRY(dmalloc(&dg, N.params * sizeof(float), "cache staging"));
    o.v.push_back(dg);
    k_unscale<<<64, 256, 0, s->stream>>>(N.g, N.params, N.scal, (float *)dg);
    KGK_CUDA(cudaGetLastError());
    KGK_CUDA(cudaMemcpyAsync(grad, dg, N.params * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    float hl = 0.0f;
    KGK_CUDA(cudaMemcpyAsync(&hl, N.scal + 1, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    KGK_CUDA(cudaStreamSynchronize(s->stream));
    if (loss) *loss = hl;
    return KGK_OK;
}

kgk_status kgk_nrc_train(kgk_scene *s, const float *raw, const float *target, size_t n, int32_t steps, float *loss) {
    KGK_TRY(need(s));
    if (!raw || !target || n == 0 || n > (1u << 30) || steps <= 0)
        return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_nrc_train: bad arguments");
    if (loss && is_device_ptr(loss)) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_nrc_train: loss must be host memory");
    Owned o;
    void *draw, *dt;
    KGK_TRY(stage_in(s, raw, n * kRaw * sizeof(float), &draw, o.v));
    KGK_TRY(stage_in(s, target, n * 3 * sizeof(float), &dt, o.v));
    NrcState &N = *s->nrc;
    for (int k = 0; k < steps; ++k) {
        KGK_TRY(nrc_grad_dev(N, (const float *)draw, kRaw, (const float *)dt, 3, (int)n, nullptr, s->stream));
        KGK_TRY(nrc_step_dev(N, s->stream));
    }
    float hl = 0.0f;
    KGK_CUDA(cudaMemcpyAsync(&hl, N.scal + 1, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
    KGK_CUDA(cudaStreamSynchronize(s->stream));
    if (loss) *loss = hl;
    return KGK_OK;
}

kgk_status kgk_nrc_loss_scale(kgk_scene *s, float *scale) {
    KGK_TRY(need(s));
    if (!scale) return fail(KGK_ERR_INVALID_ARGUMENT, "kgk_nrc_loss_scale: NULL");
    KGK_CUDA(cudaStreamSynchronize(s->stream));
    KGK_CUDA(cudaMemcpy(scale, s->nrc->scal, sizeof(float), cudaMemcpyDeviceToHost));
    return KGK_OK;
}

}  // extern "C"
