// Launcher of the persistent multi-capture gather (FP32 rows for every
// storage type), instantiated in batch_inst_f32.cu so its variants compile in
// parallel with the rest of the library.
#pragma once

#include "bp_gather.cuh"

namespace fbp {

// Voxel tile shapes the autotuner chooses from: KV voxels along x per thread,
// WY x WZ warps (each warp 8 rows x 4 depth slices).
struct TileCfg {
    int kv, wy, wz;
};
constexpr int kNumTileCfgs = 4;
constexpr TileCfg kTileCfgs[kNumTileCfgs] = {{16, 2, 4}, {8, 2, 4}, {8, 4, 4}, {4, 4, 4}};

struct BatchLaunch {
    const ConfocalGatherParams* caps;  // device
    const BatchItem* items;            // device
    uint32_t nitems;
    unsigned int* counter;             // device, zeroed before the launch
    size_t smem;       // dynamic shared memory of the launch
    int path;
    bool bounce, clamp;
    int cfg;
    size_t smem_limit;  // the kernel's dynamic shared-memory limit (set by prepare)
};

// Sets the kernel's shared-memory limit to b.smem_limit and returns the CTAs
// per SM it keeps resident with b.smem bytes each (host only; call outside
// stream capture).
template <typename S>
fbp_status batch_prepare_kernel(const BatchLaunch& b, int* ctas_per_sm);
template <typename S>
fbp_status batch_launch(fbp_context* ctx, const BatchLaunch& b, int ctas, cudaStream_t stream);

template <typename S, int KV, int WY, int WZ, int PATH, bool BOUNCE, bool CLAMP>
static fbp_status batch_variant(fbp_context* ctx, const BatchLaunch& b, int ctas, cudaStream_t stream, int* occ) {
    auto k = confocal_batch_kernel<S, KV, WY, WZ, PATH, BOUNCE, CLAMP>;
    if (occ) {
        // The opt-in limit covers static and dynamic shared memory together.
        cudaFuncAttributes fa;
        FBP_TRY_CUDA(cudaFuncGetAttributes(&fa, k));
        const size_t limit = b.smem_limit > fa.sharedSizeBytes ? b.smem_limit - fa.sharedSizeBytes : 0;
        if (b.smem > limit) return set_error(FBP_ERR_UNSUPPORTED, "batch: time-bin window too large for shared memory");
        FBP_TRY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
        FBP_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k, 32 * WY * WZ, b.smem));
        return FBP_OK;
    }
    k<<<ctas, 32 * WY * WZ, b.smem, stream>>>(b.caps, b.items, b.nitems, b.counter);
    FBP_CHECK_LAUNCH(ctx, "confocal_batch_kernel");
    return FBP_OK;
}

template <typename S, int KV, int WY, int WZ>
static fbp_status batch_dispatch_cfg(fbp_context* ctx, const BatchLaunch& b, int ctas, cudaStream_t s, int* occ) {
    if (b.path == PATH_EXACT) {
        if (b.bounce) return batch_variant<S, KV, WY, WZ, PATH_EXACT, true, true>(ctx, b, ctas, s, occ);
        return batch_variant<S, KV, WY, WZ, PATH_EXACT, false, true>(ctx, b, ctas, s, occ);
    }
    if (b.path == PATH_2D) {
        if (b.clamp) return batch_variant<S, KV, WY, WZ, PATH_2D, false, true>(ctx, b, ctas, s, occ);
        return batch_variant<S, KV, WY, WZ, PATH_2D, false, false>(ctx, b, ctas, s, occ);
    }
    if (b.bounce) {
        if (b.clamp) return batch_variant<S, KV, WY, WZ, PATH_FAST, true, true>(ctx, b, ctas, s, occ);
        return batch_variant<S, KV, WY, WZ, PATH_FAST, true, false>(ctx, b, ctas, s, occ);
    }
    if (b.clamp) return batch_variant<S, KV, WY, WZ, PATH_FAST, false, true>(ctx, b, ctas, s, occ);
    return batch_variant<S, KV, WY, WZ, PATH_FAST, false, false>(ctx, b, ctas, s, occ);
}

template <typename S>
static fbp_status batch_dispatch(fbp_context* ctx, const BatchLaunch& b, int ctas, cudaStream_t s, int* occ) {
    switch (b.cfg) {
        case 0: return batch_dispatch_cfg<S, kTileCfgs[0].kv, kTileCfgs[0].wy, kTileCfgs[0].wz>(ctx, b, ctas, s, occ);
        case 1: return batch_dispatch_cfg<S, kTileCfgs[1].kv, kTileCfgs[1].wy, kTileCfgs[1].wz>(ctx, b, ctas, s, occ);
        case 2: return batch_dispatch_cfg<S, kTileCfgs[2].kv, kTileCfgs[2].wy, kTileCfgs[2].wz>(ctx, b, ctas, s, occ);
        case 3: return batch_dispatch_cfg<S, kTileCfgs[3].kv, kTileCfgs[3].wy, kTileCfgs[3].wz>(ctx, b, ctas, s, occ);
        default: return set_error(FBP_ERR_INVALID_ARG, "batch: unknown tile configuration");
    }
}

#define FBP_INSTANTIATE_BATCH(S)                                                                  \
    template <>                                                                                   \
    fbp_status batch_prepare_kernel<S>(const BatchLaunch& b, int* ctas_per_sm) {                  \
        return batch_dispatch<S>(nullptr, b, 0, nullptr, ctas_per_sm);                            \
    }                                                                                             \
    template <>                                                                                   \
    fbp_status batch_launch<S>(fbp_context * ctx, const BatchLaunch& b, int ctas, cudaStream_t s) { \
        return batch_dispatch<S>(ctx, b, ctas, s, nullptr);                                       \
    }

}  // namespace fbp
