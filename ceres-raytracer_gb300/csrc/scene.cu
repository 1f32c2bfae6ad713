// Scene lifetime entry points of the C ABI.
#include "common.cuh"

extern "C" {

int crt_scene_create(crt_context* ctx, const crt_entity_desc* entities, uint32_t n_entities, crt_scene** out) {
    if (!ctx || !out || (n_entities && !entities)) return CRT_ERR_INVALID;
    *out = nullptr;
    crt_scene* s = new crt_scene();
    s->ctx = ctx;
    int rc = crt_guard(ctx, [&] {
        CRT_CUDA(cudaSetDevice(ctx->device));
        for (uint32_t e = 0; e < n_entities; ++e) {
            CRT_CHECK(std::isfinite(entities[e].scale) && entities[e].scale > 0, CRT_ERR_INVALID,
                      "entity scale must be a positive finite number");
            for (int k = 0; k < 3; ++k)
                CRT_CHECK(std::isfinite(entities[e].position[k]), CRT_ERR_INVALID, "entity position is not finite");
            for (int k = 0; k < 9; ++k)
                CRT_CHECK(std::isfinite(entities[e].rotation[k]), CRT_ERR_INVALID, "entity rotation is not finite");
        }
        scene_build(s, entities, n_entities);
    });
    if (rc != CRT_OK) {
        crt_scene_destroy(s);
        return rc;
    }
    *out = s;
    return CRT_OK;
}

int crt_scene_destroy(crt_scene* s) {
    if (!s) return CRT_OK;
    if (s->ctx) {
        cudaSetDevice(s->ctx->device);
        cudaStreamSynchronize(s->ctx->stream);
    }
    cudaFree(s->nodes);
    cudaFree(s->tris);
    cudaFree(s->leaf_prim);
    cudaFree(s->leaf_vn);
    cudaFree(s->leaf_entity);
    cudaFree(s->entities);
    delete s;
    return CRT_OK;
}

int crt_scene_get_stats(const crt_scene* s, crt_scene_stats* out) {
    if (!s || !out) return CRT_ERR_INVALID;
    out->n_tris = s->n_tris;
    out->n_nodes = s->n_nodes;
    out->n_entities = s->n_entities;
    out->depth = s->depth;
    out->build_ms = s->build_ms;
    out->device_bytes = s->device_bytes;
    for (int k = 0; k < 6; ++k) out->bounds[k] = s->bounds[k];
    return CRT_OK;
}

}  // extern "C"
