// Batched confocal reconstruction: many captures of uneven sizes in one
// persistent launch, optionally replayed from a captured CUDA graph, with the
// voxel tile shape chosen by timing.
//
// The reference reconstructs one capture per process run (Laser::reconstructShape,
// Laser.cu:40-67); this is the batched form of the same gather
// (fbp_backproject_confocal) for many captures:
//   * create: validate, plan the bin windows of every capture for the current
//     tile shape, allocate the batch's own buffers once (padded rows, tables,
//     parameters, work list), build the per-capture tables;
//   * run: re-prepare every capture's padded rows, reset the work counters,
//     launch one persistent kernel per arithmetic variant (normally one); CTAs
//     pull (capture, tile) items, largest captures first;
//   * graph: the run's launches are captured once into a CUDA graph and
//     replayed (no allocation or synchronisation inside the captured region);
//   * autotune: time every tile shape on this batch, keep the fastest.
#include "batch_launch.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace fbp {

// Captures that share one persistent launch: same arithmetic variant and the
// same resident CTAs per SM at their own shared-memory size (so a capture with
// a wide bin window does not lower the occupancy of the others).
struct BatchGroup {
    int path = 0;
    bool bounce = false, clamp = false;
    int occ = 0;  // CTAs per SM
    std::vector<uint32_t> captures;
    double work = 0.0;  // voxel-samples
    BatchItem* d_items = nullptr;
    uint32_t nitems = 0;
    size_t smem = 0;
    int ctas = 0;
};

constexpr int kMaxGroups = 64;
constexpr size_t kBatchStaticSmem = 64;  // at least confocal_batch_kernel's static shared memory

}  // namespace fbp

struct fbp_batch {
    fbp_context* ctx = nullptr;
    std::vector<fbp_capture_desc> caps;
    int dtype = FBP_F32;
    int cfg = 0;
    // Device buffers owned by the batch.
    void* rows = nullptr;
    size_t rows_bytes = 0;
    std::vector<size_t> rows_off;       // per capture, bytes
    float4* scan = nullptr;             // all scan tables back to back
    float* axes = nullptr;              // all axis tables back to back
    std::vector<size_t> scan_off, axes_off;
    fbp::ConfocalGatherParams* d_params = nullptr;
    fbp::BatchItem* d_items = nullptr;
    size_t items_cap = 0;
    unsigned int* d_counters = nullptr;
    std::vector<fbp::ConfocalGatherParams> params;
    std::vector<fbp::BatchGroup> groups;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_launches = 0;  // kernels one replay launches
    // Groups after the first run on side streams, forked from and joined
    // back into the caller's stream (parallel branches of a captured graph).
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
};

namespace fbp {
namespace {

int path_of(const fbp_recon_info& in) {
    if (in.time_offset > 0.f) return PATH_EXACT;
    if (in.discard_first_last_bounces != 0 && in.time_offset == 0.f) return PATH_2D;
    return PATH_FAST;
}

void drop_graph(fbp_batch* b) {
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->graph_exec = nullptr;
    b->graph = nullptr;
}

// Rows are FP32 for every storage type (16-bit captures are widened when the
// rows are made), so one set of kernels serves all of them.
constexpr size_t kRowBytes = sizeof(float);

fbp_status prepare_any(const BatchLaunch& l, int* occ) { return batch_prepare_kernel<float>(l, occ); }

fbp_status launch_any(fbp_context* ctx, const BatchLaunch& l, int ctas, cudaStream_t s) {
    return batch_launch<float>(ctx, l, ctas, s);
}

fbp_status rows_any(fbp_context* ctx, int dtype, const fbp_capture_desc& c, uint32_t pitch, void* dst,
                    cudaStream_t s) {
    const uint32_t L = c.info.num_laser_targets, T = c.info.num_time_bins;
    float* rows = static_cast<float*>(dst);
    switch (dtype) {
        case FBP_F32: return prepare_rows_into<float>(ctx, c.cube, c.layout, L, T, pitch, rows, s);
        case FBP_BF16: return prepare_rows_into<__nv_bfloat16>(ctx, c.cube, c.layout, L, T, pitch, rows, s);
        default: return prepare_rows_into<__half>(ctx, c.cube, c.layout, L, T, pitch, rows, s);
    }
}

// (Re)plan windows, parameters and work items for tile configuration `cfg`.
fbp_status plan_config(fbp_batch* b, int cfg, cudaStream_t s) {
    const TileCfg tc = kTileCfgs[cfg];
    const int align = (int)(16 / kRowBytes);
    const size_t meta = ConfocalGatherParams::meta_bytes(32) + kahan_smem_bytes(tc.kv, 32 * tc.wy * tc.wz) + 16;
    const uint32_t n = (uint32_t)b->caps.size();
    b->params.assign(n, ConfocalGatherParams{});
    b->groups.clear();
    std::vector<uint32_t> pitches(n);
    size_t rows_total = 0;
    std::vector<size_t> rows_off(n);
    for (uint32_t i = 0; i < n; ++i) {
        const fbp_recon_info& in = b->caps[i].info;
        const double ex = (double)std::min<uint32_t>(tc.kv, in.voxel_res[0]) * std::fabs(in.voxel_size[0]);
        const double ey = (double)std::min<uint32_t>(4 * tc.wz, in.voxel_res[2]) * std::fabs(in.voxel_size[1]);
        const double ez = (double)std::min<uint32_t>(8 * tc.wy, in.voxel_res[1]) * std::fabs(in.voxel_size[2]);
        WindowPlan wp;
        FBP_TRY(plan_window(b->ctx, ex, ey, ez, in.time_step, in.num_time_bins, align, kRowBytes, meta, &wp,
                            "fbp_batch"));
        // Leave room for the persistent kernel's own static shared memory
        // (replanning only the windows that fill the SM, so the others keep
        // the single-capture gather's plan).
        if (wp.smem + kBatchStaticSmem > (size_t)b->ctx->smem_optin)
            FBP_TRY(plan_window(b->ctx, ex, ey, ez, in.time_step, in.num_time_bins, align, kRowBytes,
                                meta + kBatchStaticSmem, &wp, "fbp_batch"));
        pitches[i] = wp.pitch;
        rows_off[i] = rows_total;
        rows_total += ((size_t)in.num_laser_targets * wp.pitch * kRowBytes + 255) & ~size_t(255);
        ConfocalGatherParams& p = b->params[i];
        p.scan = b->scan + b->scan_off[i];
        p.xs = b->axes + b->axes_off[i];
        p.ys = p.xs + in.voxel_res[0];
        p.zs = p.ys + in.voxel_res[2];
        p.volume = b->caps[i].volume;
        p.status = b->ctx->status_dev;
        p.Vx = in.voxel_res[0];
        p.Vy = in.voxel_res[1];
        p.Vz = in.voxel_res[2];
        p.L = in.num_laser_targets;
        p.T = in.num_time_bins;
        p.t0 = in.time_offset;
        p.dt = in.time_step;
        p.row_pitch = wp.pitch;
        p.slot_w = wp.slot_w;
        p.ch = wp.ch;
        p.exact_weights = b->ctx->weight_mode == FBP_WEIGHTS_REFERENCE;
        // Group by arithmetic variant and occupancy.
        const int path = path_of(in);
        const bool bounce = in.discard_first_last_bounces == 0;
        const bool clamp = path == PATH_EXACT || wp.capped;
        BatchLaunch probe{};
        probe.smem = wp.smem;
        probe.smem_limit = (size_t)b->ctx->smem_optin;
        probe.path = path;
        probe.bounce = bounce;
        probe.clamp = clamp;
        probe.cfg = cfg;
        int occ = 0;
        FBP_TRY(prepare_any(probe, &occ));
        if (occ < 1) return set_error(FBP_ERR_UNSUPPORTED, "fbp_batch: a capture's tile does not fit on an SM");
        BatchGroup* g = nullptr;
        for (auto& gg : b->groups)
            if (gg.path == path && gg.bounce == bounce && gg.clamp == clamp && gg.occ == occ) g = &gg;
        if (!g) {
            b->groups.push_back(BatchGroup{});
            g = &b->groups.back();
            g->path = path;
            g->bounce = bounce;
            g->clamp = clamp;
            g->occ = occ;
        }
        g->captures.push_back(i);
        g->work += (double)in.num_laser_targets * in.voxel_res[0] * in.voxel_res[1] * in.voxel_res[2];
        g->smem = std::max(g->smem, wp.smem);
    }
    if (b->groups.size() > (size_t)kMaxGroups)
        return set_error(FBP_ERR_UNSUPPORTED, "fbp_batch: too many (variant, occupancy) groups");
    // Largest group first: it starts on every SM, the others backfill.
    std::stable_sort(b->groups.begin(), b->groups.end(),
                     [](const BatchGroup& x, const BatchGroup& y) { return x.work > y.work; });
    // Rows buffer (grow only).
    if (rows_total > b->rows_bytes) {
        if (b->rows) FBP_TRY_CUDA(cudaFree(b->rows));
        b->rows = nullptr;
        FBP_TRY_CUDA(cudaMalloc(&b->rows, rows_total));
        b->rows_bytes = rows_total;
    }
    b->rows_off = rows_off;
    for (uint32_t i = 0; i < n; ++i) b->params[i].rows = static_cast<char*>(b->rows) + rows_off[i];
    // Work items, largest captures first within each group.
    size_t total_items = 0;
    std::vector<std::vector<BatchItem>> per_group(b->groups.size());
    for (size_t gi = 0; gi < b->groups.size(); ++gi) {
        auto& g = b->groups[gi];
        std::vector<uint32_t> order = g.captures;
        std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) {
            return b->caps[x].info.num_laser_targets > b->caps[y].info.num_laser_targets;
        });
        for (uint32_t c : order) {
            const fbp_recon_info& in = b->caps[c].info;
            const uint32_t gx = cdiv(in.voxel_res[0], tc.kv), gy = cdiv(in.voxel_res[1], 8 * tc.wy),
                           gz = cdiv(in.voxel_res[2], 4 * tc.wz);
            for (uint32_t z = 0; z < gz; ++z)
                for (uint32_t y = 0; y < gy; ++y)
                    for (uint32_t x = 0; x < gx; ++x) per_group[gi].push_back(BatchItem{c, x, y, z});
        }
        total_items += per_group[gi].size();
    }
    if (total_items > b->items_cap) {
        if (b->d_items) FBP_TRY_CUDA(cudaFree(b->d_items));
        b->d_items = nullptr;
        FBP_TRY_CUDA(cudaMalloc(&b->d_items, total_items * sizeof(BatchItem)));
        b->items_cap = total_items;
    }
    size_t off = 0;
    for (size_t gi = 0; gi < b->groups.size(); ++gi) {
        auto& g = b->groups[gi];
        g.d_items = b->d_items + off;
        g.nitems = (uint32_t)per_group[gi].size();
        FBP_TRY_CUDA(cudaMemcpyAsync(g.d_items, per_group[gi].data(), g.nitems * sizeof(BatchItem),
                                     cudaMemcpyHostToDevice, s));
        off += g.nitems;
    }
    FBP_TRY_CUDA(cudaMemcpyAsync(b->d_params, b->params.data(), n * sizeof(ConfocalGatherParams),
                                 cudaMemcpyHostToDevice, s));
    // Resident CTAs of each group (outside any capture), capped by its items.
    for (auto& g : b->groups) {
        BatchLaunch l{b->d_params, g.d_items, g.nitems, nullptr, g.smem, g.path, g.bounce, g.clamp, cfg,
                      (size_t)b->ctx->smem_optin};
        int occ = 0;
        FBP_TRY(prepare_any(l, &occ));
        g.ctas = (int)std::min<uint64_t>((uint64_t)std::max(1, occ) * b->ctx->sm_count, g.nitems);
    }
    // Side streams and events for the groups after the first.
    if (!b->fork) FBP_TRY_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    while (b->side.size() + 1 < b->groups.size()) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        FBP_TRY_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        b->side.push_back(st);
        FBP_TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        b->join.push_back(ev);
    }
    FBP_TRY_CUDA(cudaStreamSynchronize(s));  // host-side vectors above are temporaries
    b->cfg = cfg;
    drop_graph(b);
    return FBP_OK;
}

// The captured sequence: rows of every capture, counters, then one
// persistent launch per group, group 0 on `s` and the others on side streams
// forked from `s` after the counters are reset and joined back into it.
fbp_status enqueue_run(fbp_batch* b, cudaStream_t s) {
    for (size_t i = 0; i < b->caps.size(); ++i)
        FBP_TRY(rows_any(b->ctx, b->dtype, b->caps[i], b->params[i].row_pitch, const_cast<void*>(b->params[i].rows), s));
    FBP_TRY_CUDA(cudaMemsetAsync(b->d_counters, 0, b->groups.size() * sizeof(unsigned int), s));
    const size_t ng = b->groups.size();
    if (ng > 1) {
        FBP_TRY_CUDA(cudaEventRecord(b->fork, s));
        for (size_t gi = 1; gi < ng; ++gi) FBP_TRY_CUDA(cudaStreamWaitEvent(b->side[gi - 1], b->fork, 0));
    }
    for (size_t gi = 0; gi < ng; ++gi) {
        const auto& g = b->groups[gi];
        BatchLaunch l{b->d_params, g.d_items, g.nitems, b->d_counters + gi, g.smem, g.path, g.bounce, g.clamp, b->cfg,
                      (size_t)b->ctx->smem_optin};
        FBP_TRY(launch_any(b->ctx, l, g.ctas, gi == 0 ? s : b->side[gi - 1]));
    }
    for (size_t gi = 1; gi < ng; ++gi) {
        FBP_TRY_CUDA(cudaEventRecord(b->join[gi - 1], b->side[gi - 1]));
        FBP_TRY_CUDA(cudaStreamWaitEvent(s, b->join[gi - 1], 0));
    }
    return FBP_OK;
}

}  // namespace
}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_batch_destroy(fbp_batch* b) {
    return guarded("fbp_batch_destroy", [&]() -> fbp_status {
        clear_error();
        if (!b) return FBP_OK;
        if (b->ctx) use_device(b->ctx->device);
        cudaDeviceSynchronize();
        drop_graph(b);
        cudaFree(b->rows);
        cudaFree(b->scan);
        cudaFree(b->axes);
        cudaFree(b->d_params);
        cudaFree(b->d_items);
        cudaFree(b->d_counters);
        for (cudaStream_t st : b->side) cudaStreamDestroy(st);
        for (cudaEvent_t ev : b->join) cudaEventDestroy(ev);
        if (b->fork) cudaEventDestroy(b->fork);
        delete b;
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_batch_create(fbp_context* ctx, uint32_t n, const fbp_capture_desc* captures,
                                       fbp_batch** out) {
    return guarded("fbp_batch_create", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        if (!out || !captures || n == 0) return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_create: empty batch");
        *out = nullptr;
        const int dtype = captures[0].dtype;
        if (dtype != FBP_F32 && dtype != FBP_BF16 && dtype != FBP_F16)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_create: unknown dtype");
        for (uint32_t i = 0; i < n; ++i) {
            const fbp_capture_desc& c = captures[i];
            FBP_TRY(validate_info(&c.info, false, "fbp_batch_create"));
            if (c.dtype != dtype) return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_create: captures must share one dtype");
            if (!c.cube || !c.laser_xyz || !c.volume) return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_create: null buffer");
            if (c.layout != FBP_LAYOUT_TIME_MAJOR && c.layout != FBP_LAYOUT_TIME_INNER)
                return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_create: unknown layout");
        }
        fbp_batch* b = new (std::nothrow) fbp_batch();
        if (!b) return set_error(FBP_ERR_OOM, "fbp_batch_create: host allocation failed");
        b->ctx = ctx;
        b->caps.assign(captures, captures + n);
        b->dtype = dtype;
        auto fail = [&](fbp_status st) {
            const std::string msg = fbp_last_error();
            fbp_batch_destroy(b);
            return set_error(st, msg);
        };
        size_t scan_total = 0, axes_total = 0;
        for (uint32_t i = 0; i < n; ++i) {
            b->scan_off.push_back(scan_total);
            b->axes_off.push_back(axes_total);
            scan_total += captures[i].info.num_laser_targets;
            axes_total += (size_t)captures[i].info.voxel_res[0] + captures[i].info.voxel_res[1] + captures[i].info.voxel_res[2];
        }
        cudaStream_t s = nullptr;
        if (cudaMalloc(&b->scan, scan_total * sizeof(float4)) != cudaSuccess ||
            cudaMalloc(&b->axes, axes_total * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&b->d_params, n * sizeof(ConfocalGatherParams)) != cudaSuccess ||
            cudaMalloc(&b->d_counters, kMaxGroups * sizeof(unsigned int)) != cudaSuccess)
            return fail(set_error(FBP_ERR_OOM, "fbp_batch_create: device allocation failed"));
        for (uint32_t i = 0; i < n; ++i) {
            const fbp_recon_info& in = captures[i].info;
            float4* sc = b->scan + b->scan_off[i];
            float* ax = b->axes + b->axes_off[i];
            scan_table_kernel<<<cdiv(in.num_laser_targets, 256), 256, 0, s>>>(
                sc, captures[i].laser_xyz, in.num_laser_targets, (int)in.discard_first_last_bounces, in.laser_position[0],
                in.laser_position[1], in.laser_position[2], in.sensor_position[0], in.sensor_position[1],
                in.sensor_position[2], 1);
            const uint32_t vmax = std::max(in.voxel_res[0], std::max(in.voxel_res[1], in.voxel_res[2]));
            axis_tables_kernel<<<cdiv(vmax, 256), 256, 0, s>>>(
                ax, ax + in.voxel_res[0], ax + in.voxel_res[0] + in.voxel_res[2], in.voxel_res[0], in.voxel_res[1],
                in.voxel_res[2], in.hidden_min[0], in.hidden_min[1], in.hidden_min[2], in.voxel_size[0], in.voxel_size[1],
                in.voxel_size[2]);
            if (cudaGetLastError() != cudaSuccess) return fail(set_error(FBP_ERR_CUDA, "fbp_batch_create: table kernels"));
            ctx->launches += 2;
        }
        fbp_status st = plan_config(b, 0, s);
        if (st != FBP_OK) return fail(st);
        *out = b;
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_batch_run(fbp_batch* b, int use_graph, void* stream) {
    return guarded("fbp_batch_run", [&]() -> fbp_status {
        clear_error();
        if (!b) return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_run: null batch");
        FBP_TRY(check_ctx(b->ctx));
        cudaStream_t s = (cudaStream_t)stream;
        if (!use_graph) return enqueue_run(b, s);
        if (s == nullptr)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_run: graph replay needs a non-default stream");
        if (!b->graph_exec) {
            FBP_TRY_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            const uint64_t launches0 = b->ctx->launches;
            fbp_status st = enqueue_run(b, s);
            cudaGraph_t g = nullptr;
            const cudaError_t e = cudaStreamEndCapture(s, &g);
            if (st != FBP_OK) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (e != cudaSuccess) return cuda_error(e, "fbp_batch_run: cudaStreamEndCapture");
            b->graph = g;
            FBP_TRY_CUDA(cudaGraphInstantiate(&b->graph_exec, g, 0));
            b->graph_launches = b->ctx->launches - launches0;
            b->ctx->launches = launches0;  // captured, not launched
        }
        FBP_TRY_CUDA(cudaGraphLaunch(b->graph_exec, s));
        b->ctx->launches += b->graph_launches;
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_batch_autotune(fbp_batch* b, void* stream, int* chosen) {
    return guarded("fbp_batch_autotune", [&]() -> fbp_status {
        clear_error();
        if (!b) return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_autotune: null batch");
        FBP_TRY(check_ctx(b->ctx));
        cudaStream_t s = (cudaStream_t)stream;
        cudaEvent_t e0, e1;
        FBP_TRY_CUDA(cudaEventCreate(&e0));
        FBP_TRY_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        int best_cfg = b->cfg;
        fbp_status st = FBP_OK;
        // Each shape: one timed run; short batches are re-run until about 20 ms
        // are timed (at most 8 runs), so the cost stays near 3 runs for large
        // batches while small ones still get a stable figure.
        for (int cfg = 0; cfg < kNumTileCfgs && st == FBP_OK; ++cfg) {
            st = plan_config(b, cfg, s);
            if (st != FBP_OK) break;
            int reps = 1;
            float ms = 0.f;
            for (int round = 0; round < 2; ++round) {
                cudaEventRecord(e0, s);
                for (int r = 0; r < reps && st == FBP_OK; ++r) st = enqueue_run(b, s);
                cudaEventRecord(e1, s);
                if (st != FBP_OK) break;
                if (cudaEventSynchronize(e1) != cudaSuccess) {
                    st = set_error(FBP_ERR_CUDA, "fbp_batch_autotune: timing failed");
                    break;
                }
                cudaEventElapsedTime(&ms, e0, e1);
                ms /= (float)reps;
                if (ms >= 20.f) break;
                reps = std::min(8, (int)std::ceil(20.f / std::max(ms, 0.01f)));
            }
            if (st != FBP_OK) break;
            if (ms < best) {
                best = ms;
                best_cfg = cfg;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (st != FBP_OK) return st;
        FBP_TRY(plan_config(b, best_cfg, s));
        if (chosen) *chosen = best_cfg;
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_batch_set_config(fbp_batch* b, int config, void* stream) {
    return guarded("fbp_batch_set_config", [&]() -> fbp_status {
        clear_error();
        if (!b) return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_set_config: null batch");
        if (config < 0 || config >= kNumTileCfgs) return set_error(FBP_ERR_INVALID_ARG, "fbp_batch_set_config: bad config");
        FBP_TRY(check_ctx(b->ctx));
        return plan_config(b, config, (cudaStream_t)stream);
    });
}
