// msbfs.cu - fused multi-source traversal (64 sources per bitmask word).
#include "ptg_device.cuh"

namespace ptg {

bool msbfs_fused(ptg_graph *, const uint32_t *, uint32_t, uint32_t *, bool, uint32_t, RunResult &) {
    return false;
}

}  // namespace ptg
