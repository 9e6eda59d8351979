// Context, error reporting and the library version string.
#include "pg_internal.cuh"

#include <cstring>

static thread_local char g_last_error[512] = "";

void pg_set_last_error(cudaError_t e, const char *what, const char *file, int line)
{
    snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s:%d)", cudaGetErrorString(e), what, file, line);
}

int pg_check_launch(pg_ctx *ctx)
{
    (void)ctx;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        pg_set_last_error(e, "kernel launch", __FILE__, __LINE__);
        return PG_ERR_CUDA;
    }
    return PG_OK;
}

extern "C" const char *pg_error_string(int code)
{
    switch (code) {
    case PG_OK: return "PG_OK";
    case PG_ERR_ARG: return "PG_ERR_ARG: bad argument";
    case PG_ERR_CUDA: return g_last_error[0] ? g_last_error : "PG_ERR_CUDA: CUDA runtime failure";
    case PG_ERR_STORAGE: return "PG_ERR_STORAGE: unsupported storage";
    case PG_ERR_SHAPE: return "PG_ERR_SHAPE: extents do not match";
    case PG_ERR_NONFINITE: return "PG_ERR_NONFINITE: non-finite value";
    case PG_ERR_BREAKDOWN: return "PG_ERR_BREAKDOWN: Krylov breakdown";
    case PG_ERR_NOT_CONVERGED: return "PG_ERR_NOT_CONVERGED: iteration cap reached";
    case PG_ERR_ALLOC: return "PG_ERR_ALLOC: device allocation failed";
    case PG_ERR_STATE: return "PG_ERR_STATE: object not ready";
    default: return "unknown status";
    }
}

extern "C" const char *pg_version(void)
{
#ifndef PG_BUILD_FLAGS
#define PG_BUILD_FLAGS "unknown"
#endif
    return "libpyprop_gpu for sm_103a (" PG_BUILD_FLAGS ")";
}

extern "C" int pg_ctx_create(int device, pg_ctx **out)
{
    if (!out) return PG_ERR_ARG;
    int count = 0;
    PG_CUDA_TRY(cudaGetDeviceCount(&count));
    if (device < 0 || device >= count) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaSetDevice(device));
    pg_ctx *ctx = new pg_ctx();
    ctx->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        pg_set_last_error(e, "cudaStreamCreate", __FILE__, __LINE__);
        delete ctx;
        return PG_ERR_CUDA;
    }
    ctx->stream = ctx->own_stream;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    int st = pg_ctx_ensure_reduction(ctx);
    if (st != PG_OK) {
        pg_ctx_destroy(ctx);
        return st;
    }
    *out = ctx;
    return PG_OK;
}

int pg_ctx_ensure_reduction(pg_ctx *ctx)
{
    if (ctx->red_partial) return PG_OK;
    ctx->red_max_blocks = PG_RED_BLOCKS;
    ctx->red_max_cols = PG_RED_COLS;
    PG_CUDA_TRY(cudaMalloc(&ctx->red_partial, sizeof(double) * 2 * PG_RED_BLOCKS * PG_RED_COLS));
    PG_CUDA_TRY(cudaMalloc(&ctx->red_counter, sizeof(unsigned int) * 64));
    PG_CUDA_TRY(cudaMemset(ctx->red_counter, 0, sizeof(unsigned int) * 64));
    PG_CUDA_TRY(cudaMalloc(&ctx->red_out, sizeof(double) * 2 * PG_RED_COLS));
    PG_CUDA_TRY(cudaMallocHost(&ctx->h_pinned, sizeof(double) * 2 * PG_RED_COLS));
    PG_CUDA_TRY(cudaMalloc(&ctx->d_err, sizeof(int) * 4));
    PG_CUDA_TRY(cudaMemset(ctx->d_err, 0, sizeof(int) * 4));
    return PG_OK;
}

extern "C" int pg_ctx_destroy(pg_ctx *ctx)
{
    if (!ctx) return PG_ERR_ARG;
    if (ctx->own_stream) cudaStreamSynchronize(ctx->own_stream);
    cudaFree(ctx->red_partial);
    cudaFree(ctx->red_counter);
    cudaFree(ctx->red_out);
    cudaFree(ctx->d_err);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return PG_OK;
}

extern "C" void *pg_ctx_stream(pg_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" int pg_ctx_set_stream(pg_ctx *ctx, void *stream)
{
    if (!ctx) return PG_ERR_ARG;
    // NULL is the legacy default stream (what torch reports as stream 0), so the library's
    // kernels stay ordered with the caller's work on that stream
    ctx->stream = (cudaStream_t)stream;
    return PG_OK;
}

extern "C" int pg_ctx_use_own_stream(pg_ctx *ctx)
{
    if (!ctx) return PG_ERR_ARG;
    ctx->stream = ctx->own_stream;
    return PG_OK;
}

extern "C" long long pg_ctx_kernel_launches(pg_ctx *ctx) { return ctx ? ctx->launches : -1; }

extern "C" int pg_ctx_device_error(pg_ctx *ctx, int *flag)
{
    if (!ctx || !flag) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaMemcpyAsync(ctx->h_pinned, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    *flag = *(int *)ctx->h_pinned;
    return PG_OK;
}

extern "C" int pg_ctx_clear_device_error(pg_ctx *ctx)
{
    if (!ctx) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    return PG_OK;
}

extern "C" int pg_ctx_synchronize(pg_ctx *ctx)
{
    if (!ctx) return PG_ERR_ARG;
    PG_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return PG_OK;
}
