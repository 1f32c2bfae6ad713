// Context management, scratch memory, host/device staging and status reporting.
#include "common.cuh"

#include <cmath>
#include <cstring>

void* ctx_scratch(crt_context* ctx, ScratchSlot slot, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (ctx->scratch_bytes[slot] < bytes) {
        if (ctx->scratch[slot]) {
            CRT_CUDA(cudaStreamSynchronize(ctx->stream));
            CRT_CUDA(cudaFree(ctx->scratch[slot]));
            ctx->scratch[slot] = nullptr;
            ctx->scratch_bytes[slot] = 0;
        }
        size_t cap = bytes + bytes / 4;
        cap = (cap + 255) & ~size_t(255);
        CRT_CUDA(cudaMalloc(&ctx->scratch[slot], cap));
        ctx->scratch_bytes[slot] = cap;
    }
    return ctx->scratch[slot];
}

PinnedStaging::PinnedStaging(crt_context* c, size_t bytes) : ctx(c), slot(c->pinned_next), p(nullptr) {
    ctx->pinned_next ^= 1;
    if (!ctx->pinned_ev[slot]) CRT_CUDA(cudaEventCreateWithFlags(&ctx->pinned_ev[slot], cudaEventDisableTiming));
    CRT_CUDA(cudaEventSynchronize(ctx->pinned_ev[slot]));   // copies of this buffer's previous use
    if (ctx->pinned_bytes[slot] < bytes) {
        if (ctx->pinned[slot]) {
            CRT_CUDA(cudaFreeHost(ctx->pinned[slot]));
            ctx->pinned[slot] = nullptr;
            ctx->pinned_bytes[slot] = 0;
        }
        size_t cap = (bytes + bytes / 4 + 4095) & ~size_t(4095);
        CRT_CUDA(cudaMallocHost(&ctx->pinned[slot], cap));
        ctx->pinned_bytes[slot] = cap;
    }
    p = (char*)ctx->pinned[slot];
}

void PinnedStaging::release() {
    CRT_CUDA(cudaEventRecord(ctx->pinned_ev[slot], ctx->stream));
    released = true;
}

PinnedStaging::~PinnedStaging() {
    // every exit path, also after an error: copies already enqueued from the buffer finish before
    // its next use
    if (!released) cudaEventRecord(ctx->pinned_ev[slot], ctx->stream);
}

bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

bool is_host_mapped(const void* p) {
    if (!p) return false;
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeHost && attr.devicePointer == p;
}

const void* to_device(crt_context* ctx, const void* src, size_t bytes, ScratchSlot slot) {
    if (!src || bytes == 0) return src;
    if (is_device_ptr(src)) return src;
    void* d = ctx_scratch(ctx, slot, bytes);
    CRT_CUDA(cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return d;
}

void* out_device(crt_context* ctx, void* dst, size_t bytes, ScratchSlot slot) {
    if (!dst) return nullptr;
    if (is_device_ptr(dst)) return dst;
    return ctx_scratch(ctx, slot, bytes);
}

void* out_direct(crt_context* ctx, void* dst, size_t bytes, ScratchSlot slot) {
    if (!dst) return nullptr;
    if (is_device_ptr(dst) || is_host_mapped(dst)) return dst;
    return ctx_scratch(ctx, slot, bytes);
}

void out_finish(crt_context* ctx, void* dst, const void* staged, size_t bytes) {
    if (!dst || dst == staged || bytes == 0) return;
    CRT_CUDA(cudaMemcpyAsync(dst, staged, bytes, cudaMemcpyDeviceToHost, ctx->stream));
}

void check_launch(crt_context* ctx, const char* what) {
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw CrtError{CRT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e)};
}

void check_device_error(crt_context* ctx, const char* what) {
    uint32_t h = 0;
    CRT_CUDA(cudaMemcpyAsync(&h, ctx->d_error, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    CRT_CUDA(cudaStreamSynchronize(ctx->stream));
    if (h) {
        CRT_CUDA(cudaMemsetAsync(ctx->d_error, 0, sizeof(uint32_t), ctx->stream));
        std::string m = std::string(what) + ": device check failed (";
        if (h & DEVERR_STACK_OVERFLOW) m += " traversal-stack-overflow";
        if (h & DEVERR_BUILD_OVERFLOW) m += " build-overflow";
        if (h & DEVERR_QUANT_RANGE) m += " quantisation-range";
        if (h & DEVERR_WAIT_LIMIT) m += " wait-limit";
        if (h & DEVERR_BAD_INDEX) m += " bad-index";
        m += " )";
        throw CrtError{(h & DEVERR_WAIT_LIMIT) ? CRT_ERR_TIMEOUT : CRT_ERR_DEVICE, m};
    }
}

int occupancy_grid(crt_context* ctx, const void* kernel, int block, size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm * ctx->sm_count;
}

CamBasis make_camera_basis(const crt_camera_desc* cam) {
    // SimpleCamera::pixel_to_ray (cameras/simple_camera.hpp:61-81) is, before normalisation,
    // R^T ((u - cx)/sx, (cy - v)/sy, +-f): affine in (u, v).  Evaluate its three FP64 terms once.
    const double* R = cam->rotation;
    const double cx = cam->resolution[0] / 2.0, cy = cam->resolution[1] / 2.0;
    const double sx = cam->resolution[0] / cam->sensor_size[0], sy = cam->resolution[1] / cam->sensor_size[1];
    const double fz = cam->z_positive ? cam->focal_length : -cam->focal_length;
    const double a_cam[3] = {-cx / sx, cy / sy, fz};
    const double b_cam[3] = {1.0 / sx, 0.0, 0.0};
    const double c_cam[3] = {0.0, -1.0 / sy, 0.0};
    CamBasis cb;
    for (int k = 0; k < 3; ++k) {
        // (R^T v)_k = R[0][k] v0 + R[1][k] v1 + R[2][k] v2
        cb.a64[k] = R[k] * a_cam[0] + R[3 + k] * a_cam[1] + R[6 + k] * a_cam[2];
        cb.b64[k] = R[k] * b_cam[0] + R[3 + k] * b_cam[1] + R[6 + k] * b_cam[2];
        cb.c64[k] = R[k] * c_cam[0] + R[3 + k] * c_cam[1] + R[6 + k] * c_cam[2];
        cb.o64[k] = cam->position[k];
        cb.a[k] = (float)cb.a64[k];
        cb.b[k] = (float)cb.b64[k];
        cb.c[k] = (float)cb.c64[k];
        cb.o[k] = (float)cb.o64[k];
    }
    cb.width = (uint32_t)std::floor(cam->resolution[0]);
    cb.height = (uint32_t)std::floor(cam->resolution[1]);
    return cb;
}

extern "C" {

int crt_abi_version(void) { return CRT_ABI_VERSION; }

const char* crt_status_string(int s) {
    switch (s) {
        case CRT_OK: return "ok";
        case CRT_ERR_INVALID: return "invalid argument";
        case CRT_ERR_CUDA: return "CUDA error";
        case CRT_ERR_OOM: return "out of memory";
        case CRT_ERR_TIMEOUT: return "timeout";
        case CRT_ERR_IO: return "I/O error";
        case CRT_ERR_DEVICE: return "device-side check failed";
        case CRT_ERR_NO_DEVICE: return "no usable CUDA device";
        default: return "unknown status";
    }
}

int crt_context_create(int device, crt_context** out) {
    if (!out) return CRT_ERR_INVALID;
    *out = nullptr;
    crt_context* ctx = new crt_context();
    int rc = crt_guard(ctx, [&] {
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n == 0) {
            cudaGetLastError();
            throw CrtError{CRT_ERR_NO_DEVICE, "no CUDA device available"};
        }
        CRT_CHECK(device >= 0 && device < n, CRT_ERR_INVALID, "device index out of range");
        CRT_CUDA(cudaSetDevice(device));
        cudaDeviceProp prop;
        CRT_CUDA(cudaGetDeviceProperties(&prop, device));
        CRT_CHECK(prop.major * 10 + prop.minor == 103, CRT_ERR_NO_DEVICE,
                  "libcrt_gpu.so is built for sm_103a (GB300); this device is sm_" + std::to_string(prop.major) +
                      std::to_string(prop.minor));
        ctx->device = device;
        ctx->sm_count = prop.multiProcessorCount;
        ctx->max_threads_per_sm = prop.maxThreadsPerMultiProcessor;
        CRT_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
        ctx->stream = ctx->own_stream;
        CRT_CUDA(cudaMalloc(&ctx->d_counters, 4 * sizeof(unsigned long long)));
        CRT_CUDA(cudaMemset(ctx->d_counters, 0, 4 * sizeof(unsigned long long)));
        CRT_CUDA(cudaMalloc(&ctx->d_error, sizeof(uint32_t)));
        CRT_CUDA(cudaMemset(ctx->d_error, 0, sizeof(uint32_t)));
    });
    if (rc != CRT_OK) {
        crt_context_destroy(ctx);
        return rc;
    }
    *out = ctx;
    return CRT_OK;
}

int crt_context_destroy(crt_context* ctx) {
    if (!ctx) return CRT_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int i = 0; i < SCR_COUNT; ++i)
        if (ctx->scratch[i]) cudaFree(ctx->scratch[i]);
    for (int k = 0; k < 2; ++k) {
        if (ctx->pinned[k]) cudaFreeHost(ctx->pinned[k]);
        if (ctx->pinned_ev[k]) cudaEventDestroy(ctx->pinned_ev[k]);
    }
    if (ctx->d_counters) cudaFree(ctx->d_counters);
    if (ctx->d_error) cudaFree(ctx->d_error);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return CRT_OK;
}

int crt_context_set_stream(crt_context* ctx, void* stream) {
    if (!ctx) return CRT_ERR_INVALID;
    return crt_guard(ctx, [&] {
        CRT_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    });
}

void* crt_context_get_stream(crt_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int crt_context_synchronize(crt_context* ctx) {
    if (!ctx) return CRT_ERR_INVALID;
    return crt_guard(ctx, [&] { CRT_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

// Streaming read of a buffer with 16-byte loads that bypass L1 (ld.global.cg): four independent loads
// in flight per thread per iteration.  The XOR of everything read is stored only when it equals a
// value it never takes in practice, which keeps the loads without writing.
// `inner` passes per launch, so that a pass over a small (L2-resident) buffer is not shorter than the
// launch itself.
__global__ void __launch_bounds__(256) k_read_stream(const uint4* __restrict__ p, size_t n16, uint32_t inner,
                                                    uint32_t* __restrict__ sink) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    uint32_t acc = 0;
    for (uint32_t r = 0; r < inner; ++r) {
        size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        for (; i + 3 * stride < n16; i += 4 * stride) {
            const uint4 a = __ldcg(p + i), b = __ldcg(p + i + stride), c = __ldcg(p + i + 2 * stride),
                        d = __ldcg(p + i + 3 * stride);
            acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w ^ c.x ^ c.y ^ c.z ^ c.w ^ d.x ^ d.y ^ d.z ^ d.w;
        }
        for (; i < n16; i += stride) {
            const uint4 a = __ldcg(p + i);
            acc ^= a.x ^ a.y ^ a.z ^ a.w;
        }
    }
    if (acc == 0x9E3779B9u) sink[threadIdx.x & 31] = acc;
}

int crt_measure_read(crt_context* ctx, const void* buf, size_t bytes, uint32_t reps, double* ms_per_pass) {
    if (!ctx || !buf || !ms_per_pass || bytes < 16 || reps == 0) return CRT_ERR_INVALID;
    return crt_guard(ctx, [&] {
        CRT_CHECK(is_device_ptr(buf) && ((uintptr_t)buf & 15) == 0, CRT_ERR_INVALID,
                  "crt_measure_read needs a 16-byte aligned device buffer");
        CRT_CUDA(cudaSetDevice(ctx->device));
        uint32_t* sink = (uint32_t*)ctx_scratch(ctx, SCR_QUEUE, 256);
        const int grid = occupancy_grid(ctx, (const void*)k_read_stream, 256, 0);
        const uint4* p = (const uint4*)buf;
        const size_t n16 = bytes / 16;
        // passes per launch: at least 1 GiB read per launch
        const uint32_t inner = (uint32_t)std::max<size_t>(1, std::min<size_t>(4096, (size_t(1) << 30) / bytes));
        cudaEvent_t e0, e1;
        CRT_CUDA(cudaEventCreate(&e0));
        CRT_CUDA(cudaEventCreate(&e1));
        k_read_stream<<<grid, 256, 0, ctx->stream>>>(p, n16, 1, sink);   // warm-up pass (fills L2 for small buffers)
        check_launch(ctx, "k_read_stream");
        CRT_CUDA(cudaEventRecord(e0, ctx->stream));
        for (uint32_t r = 0; r < reps; ++r) k_read_stream<<<grid, 256, 0, ctx->stream>>>(p, n16, inner, sink);
        check_launch(ctx, "k_read_stream");
        CRT_CUDA(cudaEventRecord(e1, ctx->stream));
        CRT_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        CRT_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        ctx->launches += reps - 1;
        *ms_per_pass = ms / ((double)reps * inner);
    });
}

int crt_context_set_counting(crt_context* ctx, int enabled) {
    if (!ctx) return CRT_ERR_INVALID;
    ctx->counting = enabled != 0;
    return CRT_OK;
}

int crt_context_get_counters(crt_context* ctx, crt_counters* out) {
    if (!ctx || !out) return CRT_ERR_INVALID;
    return crt_guard(ctx, [&] {
        unsigned long long h[4] = {0, 0, 0, 0};
        CRT_CUDA(cudaMemcpyAsync(h, ctx->d_counters, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
        CRT_CUDA(cudaStreamSynchronize(ctx->stream));
        out->rays = h[0];
        out->nodes = h[1];
        out->tris = h[2];
        out->launches = ctx->launches;
        out->resolved = h[3];
    });
}

int crt_context_reset_counters(crt_context* ctx) {
    if (!ctx) return CRT_ERR_INVALID;
    return crt_guard(ctx, [&] {
        CRT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, 4 * sizeof(unsigned long long), ctx->stream));
        ctx->launches = 0;
    });
}

int crt_context_set_tuning(crt_context* ctx, const crt_tuning* t) {
    if (!ctx || !t) return CRT_ERR_INVALID;
    if (t->queue_chunk < 1 || t->queue_chunk > 8 || t->wave_paths < (1u << 16) ||
        !(t->collapse_tri_cost >= 0.01f && t->collapse_tri_cost <= 10.0f) || t->treelet_passes > 8) {
        ctx->last_error = "tuning out of range (queue_chunk 1..8, wave_paths >= 65536, collapse_tri_cost 0.01..10, "
                          "treelet_passes 0..8)";
        return CRT_ERR_INVALID;
    }
    ctx->queue_chunk = t->queue_chunk;
    ctx->wave_paths = t->wave_paths;
    ctx->use_graphs = t->use_graphs ? 1 : 0;
    ctx->build_sah = t->build_sah ? 1 : 0;
    ctx->collapse_tri_cost = t->collapse_tri_cost;
    ctx->treelet_passes = t->treelet_passes;
    return CRT_OK;
}

int crt_context_get_tuning(const crt_context* ctx, crt_tuning* out) {
    if (!ctx || !out) return CRT_ERR_INVALID;
    out->queue_chunk = ctx->queue_chunk;
    out->wave_paths = ctx->wave_paths;
    out->use_graphs = ctx->use_graphs;
    out->build_sah = ctx->build_sah;
    out->collapse_tri_cost = ctx->collapse_tri_cost;
    out->treelet_passes = ctx->treelet_passes;
    return CRT_OK;
}

int crt_host_alloc(size_t bytes, void** out) {
    if (!out) return CRT_ERR_INVALID;
    *out = nullptr;
    if (cudaMallocHost(out, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return CRT_ERR_OOM;
    }
    return CRT_OK;
}

int crt_host_free(void* ptr) {
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) {
        cudaGetLastError();
        return CRT_ERR_CUDA;
    }
    return CRT_OK;
}

const char* crt_context_last_error(const crt_context* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

}  // extern "C"
