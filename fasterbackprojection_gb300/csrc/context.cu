// Context, error reporting and scratch management for libfbp.
#include "fbp_internal.cuh"

#include <cstdio>
#include <cstring>

namespace fbp {

namespace {
thread_local std::string t_last_error;
thread_local int t_caller_device = -1;  // the caller's device while a call runs on another
}

fbp_status set_error(fbp_status st, const std::string& msg) {
    t_last_error = msg;
    return st;
}

fbp_status cuda_error(cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return set_error(FBP_ERR_OOM, m);
    return set_error(FBP_ERR_CUDA, m);
}

void clear_error() { t_last_error.clear(); }

fbp_status fail_quietly(fbp_status st, const char* who, const char* what) noexcept {
    try {
        t_last_error = std::string(who) + ": " + what;
    } catch (...) {  // no memory for the message: keep the status
    }
    return st;
}

fbp_status use_device(int device) {
    int cur = -1;
    FBP_TRY_CUDA(cudaGetDevice(&cur));
    if (cur != device) {
        FBP_TRY_CUDA(cudaSetDevice(device));
        if (t_caller_device < 0) t_caller_device = cur;
    }
    return FBP_OK;
}

fbp_status check_ctx(fbp_context* ctx) {
    if (!ctx) return set_error(FBP_ERR_INVALID_ARG, "null context");
    return use_device(ctx->device);
}

void restore_device() noexcept {
    if (t_caller_device >= 0) {
        cudaSetDevice(t_caller_device);
        t_caller_device = -1;
    }
}

fbp_status workspace(fbp_context* ctx, int slot, size_t bytes, cudaStream_t stream, void** out) {
    if (slot < 0 || slot >= WS_NUM_SLOTS) return set_error(FBP_ERR_INVALID_ARG, "bad workspace slot");
    if (bytes == 0) bytes = 16;
    if (ctx->ws_bytes[slot] < bytes) {
        if (ctx->ws[slot]) {
            // Kernels queued earlier on this stream may still read the old buffer.
            FBP_TRY_CUDA(cudaStreamSynchronize(stream));
            FBP_TRY_CUDA(cudaFree(ctx->ws[slot]));
            ctx->ws[slot] = nullptr;
            ctx->ws_bytes[slot] = 0;
        }
        const size_t rounded = (bytes + 255) & ~size_t(255);
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, rounded);
        if (e != cudaSuccess) return cuda_error(e, "workspace cudaMalloc");
        ctx->ws[slot] = p;
        ctx->ws_bytes[slot] = rounded;
    }
    *out = ctx->ws[slot];
    return FBP_OK;
}

}  // namespace fbp

using namespace fbp;

extern "C" {

const char* fbp_version(void) { return "fbp-gb300 1.0 (sm_103a)"; }

const char* fbp_last_error(void) { return t_last_error.c_str(); }

fbp_status fbp_create(fbp_context** out, int device) {
    return guarded("fbp_create", [&]() -> fbp_status {
        clear_error();
        if (!out) return set_error(FBP_ERR_INVALID_ARG, "fbp_create: null output pointer");
        *out = nullptr;
        int n = 0;
        FBP_TRY_CUDA(cudaGetDeviceCount(&n));
        if (device < 0 || device >= n) return set_error(FBP_ERR_INVALID_ARG, "fbp_create: no such device");
        FBP_TRY(use_device(device));
        cudaDeviceProp prop;
        FBP_TRY_CUDA(cudaGetDeviceProperties(&prop, device));
        if (prop.major < 10) return set_error(FBP_ERR_UNSUPPORTED, "fbp_create: libfbp is built for sm_103a (GB300)");
        fbp_context* ctx = new (std::nothrow) fbp_context();
        if (!ctx) return set_error(FBP_ERR_OOM, "fbp_create: host allocation failed");
        ctx->device = device;
        ctx->sm_count = prop.multiProcessorCount;
        ctx->smem_optin = (int)prop.sharedMemPerBlockOptin;
        cudaError_t e = cudaMalloc(&ctx->status_dev, sizeof(int));
        if (e == cudaSuccess) e = cudaMemset(ctx->status_dev, 0, sizeof(int));
        if (e != cudaSuccess) {
            cudaFree(ctx->status_dev);
            delete ctx;
            return cuda_error(e, "fbp_create: status word");
        }
        *out = ctx;
        return FBP_OK;
    });
}

fbp_status fbp_destroy(fbp_context* ctx) {
    return guarded("fbp_destroy", [&]() -> fbp_status {
        clear_error();
        if (!ctx) return FBP_OK;
        use_device(ctx->device);
        cudaDeviceSynchronize();
        for (int i = 0; i < WS_NUM_SLOTS; ++i)
            if (ctx->ws[i]) cudaFree(ctx->ws[i]);
        for (void* t : ctx->twiddles)
            if (t) cudaFree(t);
        for (void* t : ctx->stage_twiddles)
            if (t) cudaFree(t);
        if (ctx->status_dev) cudaFree(ctx->status_dev);
        delete ctx;
        return FBP_OK;
    });
}

fbp_status fbp_check_device_status(fbp_context* ctx, void* stream) {
    return guarded("fbp_check_device_status", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        cudaStream_t s = (cudaStream_t)stream;
        int h = 0;
        FBP_TRY_CUDA(cudaMemcpyAsync(&h, ctx->status_dev, sizeof(int), cudaMemcpyDeviceToHost, s));
        FBP_TRY_CUDA(cudaMemsetAsync(ctx->status_dev, 0, sizeof(int), s));
        FBP_TRY_CUDA(cudaStreamSynchronize(s));
        if (h == 0) return FBP_OK;
        char buf[96];
        snprintf(buf, sizeof(buf), "device status word reported %d", h);
        return set_error(h == FBP_ERR_TIMEOUT ? FBP_ERR_TIMEOUT : FBP_ERR_DEVICE, buf);
    });
}

uint64_t fbp_kernel_launch_count(const fbp_context* ctx) { return ctx ? ctx->launches : 0; }

extern "C" fbp_status fbp_set_weight_mode(fbp_context* ctx, int mode) {
    clear_error();
    if (!ctx) return set_error(FBP_ERR_INVALID_ARG, "fbp_set_weight_mode: null context");
    if (mode != FBP_WEIGHTS_BATCHED && mode != FBP_WEIGHTS_REFERENCE)
        return set_error(FBP_ERR_INVALID_ARG, "fbp_set_weight_mode: unknown mode");
    ctx->weight_mode = mode;
    return FBP_OK;
}

extern "C" fbp_status fbp_get_weight_mode(const fbp_context* ctx, int* mode) {
    clear_error();
    if (!ctx || !mode) return set_error(FBP_ERR_INVALID_ARG, "fbp_get_weight_mode: null argument");
    *mode = ctx->weight_mode;
    return FBP_OK;
}

fbp_status fbp_linear_space(double min_value, double max_value, int n, double* out) {
    return guarded("fbp_linear_space", [&]() -> fbp_status {
        clear_error();
        if (n <= 0 || !out) return set_error(FBP_ERR_INVALID_ARG, "fbp_linear_space: n must be > 0 and out non-null");
        // Laser.cu:69-78: step = (max - min) / n, v[i] = min + step * i.
        const double step = (max_value - min_value) / (double)n;
        for (int i = 0; i < n; ++i) out[i] = min_value + step * i;
        return FBP_OK;
    });
}

}  // extern "C"
