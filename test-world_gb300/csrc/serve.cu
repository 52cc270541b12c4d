// serve.cu - request server (continuous batching); see ptgraph.h.
#include "ptg_device.cuh"

extern "C" {
ptg_status ptg_server_create(ptg_ctx *, const ptg_server_config *, ptg_server **out) {
    if (out) *out = nullptr;
    return PTG_ERR_UNSUPPORTED;
}
void ptg_server_destroy(ptg_server *) {}
ptg_status ptg_server_add_graph(ptg_server *, ptg_graph *, uint32_t *) { return PTG_ERR_UNSUPPORTED; }
ptg_status ptg_server_submit(ptg_server *, uint32_t, uint32_t, uint32_t, void *, uint64_t *) {
    return PTG_ERR_UNSUPPORTED;
}
ptg_status ptg_server_wait(ptg_server *, uint64_t, int64_t, double *) { return PTG_ERR_UNSUPPORTED; }
ptg_status ptg_server_drain(ptg_server *) { return PTG_ERR_UNSUPPORTED; }
ptg_status ptg_server_stats_get(ptg_server *, ptg_server_stats *) { return PTG_ERR_UNSUPPORTED; }
}
