// ref_harness.cpp - drives the reference's own kernels (ptGraph/gpu_kernels.cu,
// compiled for the host with ref_shim.h) through restatements of the
// reference's host loops in ptGraph/main.cu.  TEST INFRASTRUCTURE ONLY: it
// produces the golden fixtures under tests/golden/ that pin the C oracle.
//
// Each ref_* driver below follows one reference entry point step by step:
// the same kernels in the same order with the same arguments, the same
// <<<56, 1024>>> launch shape, Thrust's reduce/exclusive_scan replaced by
// std::accumulate/std::exclusive_scan, cudaMemcpy by memcpy, and the CPU
// gather workers (main.cu:188-220, 642-676, 1126-1156) by the same copy
// loop.  Launches are emulated by calling the kernel once per (block, thread)
// in order, so a run is one legal interleaving of the reference's threads.
//
// Deviations, all forced by undefined behaviour in the reference:
//  * the offsets array gets a sentinel offsets[n] = m, because the Opt
//    drivers read nodePointersI[maxPartitionNode + 1] with maxPartitionNode
//    = n - 1 when everything fits (main.cu:276, 731, 1232, 1462);
//  * the cut search `for (uint i = n - 1; i >= 0; i--)` (main.cu:269, 722,
//    1225, 1455) never terminates when no offset is below the budget; the
//    drivers reject such budgets instead (return -2).
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "gpu_kernels.cuh"

thread_local ptg_emu_dim3 threadIdx, blockIdx, blockDim, gridDim;

namespace {

const unsigned GRID = 56, BLOCK = 1024;  // main.cu:318-319 and every driver

template <class F>
void launch(F &&kernel_call) {
    gridDim = {GRID, 1, 1};
    blockDim = {BLOCK, 1, 1};
    for (unsigned b = 0; b < GRID; b++) {
        blockIdx = {b, 0, 0};
        for (unsigned t = 0; t < BLOCK; t++) {
            threadIdx = {t, 0, 0};
            kernel_call();
        }
    }
}

uint32_t reduce_u32(const uint32_t *p, uint32_t k) {
    return std::accumulate(p, p + k, 0u);
}

void exclusive_scan_u32(const uint32_t *in, uint32_t k, uint32_t *out) {
    std::exclusive_scan(in, in + k, out, 0u);
}

struct Csr {
    uint32_t n, m;
    std::vector<uint32_t> ptr;  // n + 1 (sentinel added)
    std::vector<uint32_t> degree;
};

Csr make_csr(uint32_t n, uint32_t m, const uint32_t *off_n) {
    Csr c;
    c.n = n;
    c.m = m;
    c.ptr.assign(off_n, off_n + n);
    c.ptr.push_back(m);
    c.degree.resize(n);
    // main.cu:1213-1220
    for (uint32_t i = 0; i + 1 < n; i++) c.degree[i] = c.ptr[i + 1] - c.ptr[i];
    c.degree[n - 1] = m - c.ptr[n - 1];
    return c;
}

// maxPartitionNode search of main.cu:1222-1232 (also 266-276, 719-731,
// 1452-1462).  Returns false when the reference loop would not terminate.
bool cut_vertex(const Csr &c, uint64_t max_partition_size, int &maxPartitionNode) {
    maxPartitionNode = (int)c.n - 1;
    if (max_partition_size < c.m) {
        bool found = false;
        for (int64_t i = (int64_t)c.n - 1; i >= 0; i--) {
            if (c.ptr[i] < max_partition_size) {
                maxPartitionNode = (int)i - 1;
                found = true;
                break;
            }
        }
        if (!found) return false;
    }
    return true;
}

// bfsDynamic / ccDynamic / ssspDynamic gather (main.cu:1147-1155): copy the
// adjacency of active overload vertices into the compacted buffer.
template <class E>
void gather(uint32_t begin, uint32_t end, const uint32_t *degree, const uint32_t *activePtr,
            const uint32_t *nodePointer, const uint32_t *activeNodes, E *overload, const E *edges) {
    for (uint32_t i = begin; i < end; i++) {
        uint32_t v = activeNodes[i];
        for (uint32_t j = 0; j < degree[v]; j++) overload[activePtr[i] + j] = edges[nodePointer[v] + j];
    }
}

// ---------------------------------------------------------------------------
// UM-only drivers: bfsCaculateInShare (main.cu:1041-1123), ssspCaculateInShare
// (563-638), ccCaculateInShare (961-1035), caculateInCommon (2396-2477).
// kind: 0 bfs, 1 sssp, 2 cc
// ---------------------------------------------------------------------------
int run_share(int kind, const Csr &c, uint32_t *edges, EdgeWithWeight *wedges, uint32_t src,
              uint32_t *value, uint32_t *iters_out) {
    uint32_t n = c.n;
    std::vector<uint8_t> labelv(n);
    bool *label = reinterpret_cast<bool *>(labelv.data());
    std::vector<uint32_t> degree = c.degree, ptr = c.ptr;
    for (uint32_t i = 0; i < n; i++) {
        if (kind == 2) {
            label[i] = true;  // main.cu:977-980
            value[i] = i;
        } else {
            label[i] = false;
            value[i] = kind == 1 ? UINT_MAX - 1 : UINT_MAX;  // main.cu:584, 1068
        }
    }
    if (kind != 2) {
        label[src] = true;
        value[src] = 1;
    }
    std::vector<uint32_t> activeNodeList(n), labeling(n), prefix(n);
    launch([&] { setLabeling(n, label, labeling.data()); });
    uint32_t activeNodesNum = reduce_u32(labeling.data(), n);
    uint32_t iter = 0;
    while (activeNodesNum > 0) {
        iter++;
        exclusive_scan_u32(labeling.data(), n, prefix.data());
        launch([&] { setActiveNodeArray(n, activeNodeList.data(), label, prefix.data()); });
        launch([&] { setLabelDefault(activeNodesNum, activeNodeList.data(), label); });
        if (kind == 0)
            launch([&] {
                bfs_kernel(activeNodesNum, activeNodeList.data(), ptr.data(), degree.data(), edges,
                           value, label);
            });
        else if (kind == 1)
            launch([&] {
                sssp_kernel(activeNodesNum, activeNodeList.data(), ptr.data(), degree.data(), wedges,
                            value, label);
            });
        else
            launch([&] {
                cc_kernel(activeNodesNum, activeNodeList.data(), ptr.data(), degree.data(), edges,
                          value, label);
            });
        launch([&] { setLabeling(n, label, labeling.data()); });
        activeNodesNum = reduce_u32(labeling.data(), n);
    }
    *iters_out = iter;
    return 0;
}

// ---------------------------------------------------------------------------
// Out-of-core drivers: bfsCaculateInOpt (main.cu:1180-1418), ssspCaculateInOpt
// (678-889), ccCaculateInOpt (222-440).  max_partition_size is the edge
// budget the reference derives from totalGlobalMem (main.cu:1193).
// ---------------------------------------------------------------------------
template <class E>
int run_opt(int kind, const Csr &c, E *edgeList, uint64_t max_partition_size, uint32_t src,
            uint32_t *value, uint32_t *iters_out) {
    uint32_t n = c.n, m = c.m;
    std::vector<uint32_t> degree = c.degree, nodePointersI = c.ptr;
    int maxPartitionNode;
    if (!cut_vertex(c, max_partition_size, maxPartitionNode)) return -2;
    max_partition_size = nodePointersI[maxPartitionNode + 1];
    std::vector<E> edgeListD(edgeList, edgeList + max_partition_size);
    std::vector<uint8_t> labelv(n);
    bool *labelD = reinterpret_cast<bool *>(labelv.data());
    for (uint32_t i = 0; i < n; i++) {
        if (kind == 2) {
            labelD[i] = true;  // main.cu:283-286
            value[i] = i;
        } else {
            labelD[i] = false;  // main.cu:740-746, 1239-1246
            value[i] = UINT_MAX;
        }
    }
    if (kind != 2) {
        labelD[src] = true;
        value[src] = 1;
    }
    std::vector<E> edgeListOverload(std::max<uint64_t>(1, m - max_partition_size));
    std::vector<uint32_t> activeNodeListD(n), labeling(n), prefix(n), overloadDegree(n),
        overloadPrefix(n), activeNodeList(n), activeOverloadNodePointers(n);
    launch([&] { setLabeling(n, labelD, labeling.data()); });
    uint32_t activeNodesNum = reduce_u32(labeling.data(), n);
    uint32_t iter = 0;
    while (activeNodesNum > 0) {
        iter++;
        exclusive_scan_u32(labeling.data(), n, prefix.data());
        launch([&] {
            setActiveNodeArrayAndNodePointer(n, activeNodeListD.data(), overloadDegree.data(), labelD,
                                             prefix.data(), (uint32_t)maxPartitionNode,
                                             degree.data());
        });
        uint32_t overloadEdgeNum = reduce_u32(overloadDegree.data(), activeNodesNum);
        exclusive_scan_u32(overloadDegree.data(), activeNodesNum, overloadPrefix.data());
        if (overloadEdgeNum > 0) {
            std::memcpy(activeNodeList.data(), activeNodeListD.data(), activeNodesNum * 4);
            std::memcpy(activeOverloadNodePointers.data(), overloadPrefix.data(), activeNodesNum * 4);
            int overloadNodeBegin = -1;
            for (uint32_t i = 0; i < activeNodesNum; i++) {
                if (activeNodeList[i] > (uint32_t)maxPartitionNode) {
                    overloadNodeBegin = (int)i;
                    break;
                }
            }
            if (overloadNodeBegin >= 0)
                gather(overloadNodeBegin, activeNodesNum, degree.data(),
                       activeOverloadNodePointers.data(), nodePointersI.data(), activeNodeList.data(),
                       edgeListOverload.data(), edgeList);
        }
        launch([&] { setLabelDefault(activeNodesNum, activeNodeListD.data(), labelD); });
        if constexpr (std::is_same<E, EdgeWithWeight>::value) {
            launch([&] {
                sssp_kernelOpt(activeNodesNum, activeNodeListD.data(), nodePointersI.data(),
                               degree.data(), edgeListD.data(), value, labelD,
                               (uint32_t)maxPartitionNode, edgeListOverload.data(),
                               overloadPrefix.data());
            });
        } else if (kind == 0) {
            launch([&] {
                bfs_kernelOpt(activeNodesNum, activeNodeListD.data(), nodePointersI.data(),
                              degree.data(), edgeListD.data(), value, labelD,
                              (uint32_t)maxPartitionNode, edgeListOverload.data(),
                              overloadPrefix.data());
            });
        } else {
            launch([&] {
                cc_kernelOpt(activeNodesNum, activeNodeListD.data(), nodePointersI.data(),
                             degree.data(), edgeListD.data(), value, labelD,
                             (uint32_t)maxPartitionNode, edgeListOverload.data(),
                             overloadPrefix.data());
            });
        }
        launch([&] { setLabeling(n, labelD, labeling.data()); });
        activeNodesNum = reduce_u32(labeling.data(), n);
    }
    *iters_out = iter;
    return 0;
}

// bfsCaculateInAsync (main.cu:1420-1678): static prefix kernel on one stream,
// dynamic (overload) kernel on the default stream after the host gather.
int run_bfs_async(const Csr &c, uint32_t *edgeList, uint64_t max_partition_size, uint32_t src,
                  uint32_t *value, uint32_t *iters_out) {
    uint32_t n = c.n, m = c.m;
    std::vector<uint32_t> degree = c.degree, nodePointersI = c.ptr;
    int maxPartitionNode;
    if (!cut_vertex(c, max_partition_size, maxPartitionNode)) return -2;
    max_partition_size = nodePointersI[maxPartitionNode + 1];
    std::vector<uint32_t> edgeListD(edgeList, edgeList + max_partition_size);
    std::vector<uint32_t> isActiveD(n, 0);
    for (uint32_t i = 0; i < n; i++) value[i] = UINT_MAX;
    isActiveD[src] = 1;
    value[src] = 1;
    std::vector<uint32_t> edgeListOverload(std::max<uint64_t>(1, m - max_partition_size));
    std::vector<uint32_t> activeNodeListD(n), prefix(n), overloadDegree(n), overloadPrefix(n),
        activeNodeList(n), activeOverloadNodePointers(n);
    uint32_t activeNodesNum = reduce_u32(isActiveD.data(), n);
    uint32_t iter = 0;
    while (activeNodesNum > 0) {
        iter++;
        exclusive_scan_u32(isActiveD.data(), n, prefix.data());
        launch([&] {
            setActiveNodeArrayAndNodePointerOpt(n, activeNodeListD.data(), overloadDegree.data(),
                                                isActiveD.data(), prefix.data(),
                                                (uint32_t)maxPartitionNode, degree.data());
        });
        uint32_t overloadNodeNum = reduce_u32(isActiveD.data(), n);
        uint32_t overloadEdgeNum = reduce_u32(overloadDegree.data(), activeNodesNum);
        exclusive_scan_u32(overloadDegree.data(), activeNodesNum, overloadPrefix.data());
        launch([&] { setLabelDefaultOpt(activeNodesNum, activeNodeListD.data(), isActiveD.data()); });
        launch([&] {
            bfs_kernelStatic(activeNodesNum - overloadNodeNum, activeNodeListD.data(),
                             nodePointersI.data(), degree.data(), edgeListD.data(), value,
                             isActiveD.data());
        });
        if (overloadEdgeNum > 0) {
            std::memcpy(activeNodeList.data(), activeNodeListD.data(), activeNodesNum * 4);
            std::memcpy(activeOverloadNodePointers.data(), overloadPrefix.data(), activeNodesNum * 4);
            int overloadNodeBegin = -1;
            for (uint32_t i = 0; i < activeNodesNum; i++) {
                if (activeNodeList[i] > (uint32_t)maxPartitionNode) {
                    overloadNodeBegin = (int)i;
                    break;
                }
            }
            if (overloadNodeBegin >= 0)
                gather<uint32_t>(overloadNodeBegin, activeNodesNum, degree.data(),
                                 activeOverloadNodePointers.data(), nodePointersI.data(),
                                 activeNodeList.data(), edgeListOverload.data(), edgeList);
            launch([&] {
                bfs_kernelDynamic(activeNodesNum, activeNodeListD.data(), degree.data(), value,
                                  isActiveD.data(), overloadNodeNum, edgeListOverload.data(),
                                  overloadPrefix.data());
            });
        }
        activeNodesNum = reduce_u32(isActiveD.data(), n);
    }
    *iters_out = iter;
    return 0;
}

// bfsCaculateInAsyncSwap (main.cu:1681-2059) with its fragment bookkeeping;
// the commented-out swap loop (main.cu:1955-2003) is not part of it.
int run_bfs_async_swap(const Csr &c, uint32_t *edgeList, uint64_t max_partition_size,
                       uint32_t fragment_size, uint32_t src, uint32_t *value, uint32_t *iters_out) {
    uint32_t n = c.n, m = c.m;
    std::vector<uint32_t> degree = c.degree, nodePointersI = c.ptr;
    max_partition_size -= max_partition_size % fragment_size;  // main.cu:1700-1701
    if (max_partition_size > m) max_partition_size = m;
    std::vector<uint32_t> edgeListD(edgeList, edgeList + max_partition_size);
    std::vector<uint8_t> isInStaticv(n);
    bool *isInStatic = reinterpret_cast<bool *>(isInStaticv.data());
    std::vector<uint32_t> isActiveD(n, 0);
    for (uint32_t i = 0; i < n; i++) {
        value[i] = UINT_MAX;
        // main.cu:1759-1764 (unsigned arithmetic as in the reference)
        isInStatic[i] = nodePointersI[i] < max_partition_size &&
                        (uint32_t)(nodePointersI[i] + degree[i] - 1) < max_partition_size;
    }
    uint32_t staticFragmentNum = (uint32_t)(max_partition_size / fragment_size);
    std::vector<uint32_t> canSwap(std::max(1u, staticFragmentNum), 0),
        canSwapPrefix(std::max(1u, staticFragmentNum)), staticFragmentDataD(std::max(1u, staticFragmentNum));
    isActiveD[src] = 1;
    value[src] = 1;
    std::vector<uint32_t> edgeListOverload(std::max<uint64_t>(1, m - max_partition_size));
    std::vector<uint32_t> activeNodeListD(n), prefix(n), overloadDegree(n), overloadPrefix(n),
        overloadNodeListD(n), overloadNodeList(n), activeOverloadNodePointers(n);
    uint32_t activeNodesNum = reduce_u32(isActiveD.data(), n);
    uint32_t iter = 0;
    while (activeNodesNum > 0) {
        iter++;
        exclusive_scan_u32(isActiveD.data(), n, prefix.data());
        launch([&] {
            setActiveNodeArrayAndNodePointerSwap(n, activeNodeListD.data(), isActiveD.data(),
                                                 prefix.data(), isInStatic);
        });
        launch([&] {
            setFragmentData(activeNodesNum, activeNodeListD.data(), nodePointersI.data(),
                            canSwap.data(), staticFragmentNum, fragment_size, isInStatic);
        });
        uint32_t canSwapFragmentNum = reduce_u32(canSwap.data(), staticFragmentNum);
        if (canSwapFragmentNum > 0) {
            exclusive_scan_u32(canSwap.data(), staticFragmentNum, canSwapPrefix.data());
            launch([&] {
                setStaticFragmentData(staticFragmentNum, canSwap.data(), canSwapPrefix.data(),
                                      staticFragmentDataD.data());
            });
        }
        uint32_t overloadNodeNum = reduce_u32(isActiveD.data(), n);
        exclusive_scan_u32(isActiveD.data(), n, prefix.data());
        launch([&] {
            setOverloadNodePointerSwap(n, overloadNodeListD.data(), overloadDegree.data(),
                                       isActiveD.data(), prefix.data(), degree.data());
        });
        exclusive_scan_u32(overloadDegree.data(), overloadNodeNum, overloadPrefix.data());
        launch([&] { setLabelDefaultOpt(activeNodesNum, activeNodeListD.data(), isActiveD.data()); });
        launch([&] {
            bfs_kernelStaticSwap(activeNodesNum, activeNodeListD.data(), nodePointersI.data(),
                                 degree.data(), edgeListD.data(), value, isActiveD.data(), isInStatic);
        });
        if (overloadNodeNum > 0) {
            std::memcpy(overloadNodeList.data(), overloadNodeListD.data(), overloadNodeNum * 4);
            std::memcpy(activeOverloadNodePointers.data(), overloadPrefix.data(), overloadNodeNum * 4);
            gather<uint32_t>(0, overloadNodeNum, degree.data(), activeOverloadNodePointers.data(),
                             nodePointersI.data(), overloadNodeList.data(), edgeListOverload.data(),
                             edgeList);
            launch([&] {
                bfs_kernelDynamicSwap(overloadNodeNum, overloadNodeListD.data(), degree.data(), value,
                                      isActiveD.data(), edgeListOverload.data(), overloadPrefix.data());
            });
        }
        activeNodesNum = reduce_u32(isActiveD.data(), n);
    }
    *iters_out = iter;
    return 0;
}

// caculateInShareOpt (main.cu:2061-2185): UM list for vertices >= cut, HBM
// prefix below it; the source is the first vertex of degree > 1000.
int run_bfs_share_opt(const Csr &c, uint32_t *edgeList, uint64_t max_partition_size,
                      uint32_t *value, uint32_t *src_out, uint32_t *iters_out) {
    uint32_t n = c.n, m = c.m;
    std::vector<uint32_t> degree(n), nodePointersI = c.ptr;
    int maxPartitionNode;
    if (!cut_vertex(c, max_partition_size, maxPartitionNode)) return -2;
    uint32_t sourceCode = 0;
    for (uint32_t i = 0; i + 1 < n; i++) {
        degree[i] = nodePointersI[i + 1] - nodePointersI[i];
        if (sourceCode == 0 && degree[i] > 1000) sourceCode = i;
    }
    degree[n - 1] = m - nodePointersI[n - 1];
    uint64_t copy = std::min<uint64_t>(max_partition_size, m);
    std::vector<uint32_t> edgeListD(edgeList, edgeList + copy);
    edgeListD.resize(std::max<uint64_t>(1, max_partition_size), 0);
    std::vector<uint8_t> labelv(n, 0);
    bool *label = reinterpret_cast<bool *>(labelv.data());
    for (uint32_t i = 0; i < n; i++) value[i] = UINT_MAX;
    label[sourceCode] = true;
    value[sourceCode] = 1;
    std::vector<uint32_t> activeNodeList(n), labeling(n), prefix(n);
    launch([&] { setLabeling(n, label, labeling.data()); });
    uint32_t activeNodesNum = reduce_u32(labeling.data(), n);
    uint32_t iter = 0;
    while (activeNodesNum > 0) {
        iter++;
        exclusive_scan_u32(labeling.data(), n, prefix.data());
        launch([&] { setActiveNodeArray(n, activeNodeList.data(), label, prefix.data()); });
        launch([&] { setLabelDefault(activeNodesNum, activeNodeList.data(), label); });
        launch([&] {
            bfs_kernelShareOpt(activeNodesNum, activeNodeList.data(), nodePointersI.data(),
                               degree.data(), edgeListD.data(), edgeList, value, label,
                               (uint32_t)maxPartitionNode);
        });
        launch([&] { setLabeling(n, label, labeling.data()); });
        activeNodesNum = reduce_u32(labeling.data(), n);
    }
    *src_out = sourceCode;
    *iters_out = iter;
    return 0;
}

// caculateInOptChooseByDegree (main.cu:2196-2394): the highest-degree
// vertices' adjacency is packed into the HBM list, the rest gathered per round.
int run_bfs_by_degree(const Csr &c, uint32_t *edgeList, uint64_t max_partition_size, uint32_t src,
                      uint32_t *value, uint32_t *iters_out) {
    uint32_t n = c.n, m = c.m;
    std::vector<uint32_t> degree = c.degree, nodePointersI = c.ptr;
    struct SortItem {
        uint32_t index;
        int degree;
    };
    std::vector<SortItem> sortedData(n);
    for (uint32_t i = 0; i < n; i++) sortedData[i] = {i, (int)degree[i]};
    // main.cu:2242 uses std::sort with a strict ">" comparator; ties are in
    // unspecified order there too, and the results do not depend on it.
    std::stable_sort(sortedData.begin(), sortedData.end(),
                     [](const SortItem &a, const SortItem &b) { return a.degree > b.degree; });
    std::vector<uint32_t> edgeListGpu(std::max<uint64_t>(1, max_partition_size), 0);
    std::vector<uint32_t> ptrOfEdgeListGpu(n, 0);
    std::vector<uint8_t> isInListv(n, 0);
    bool *isInList = reinterpret_cast<bool *>(isInListv.data());
    uint64_t edgeSum = 0, tempIndex = 0;
    for (uint32_t i = 0; i < n; i++) {
        edgeSum += sortedData[i].degree;
        if (edgeSum > max_partition_size) break;
        isInList[sortedData[i].index] = true;
        ptrOfEdgeListGpu[sortedData[i].index] = (uint32_t)tempIndex;
        for (int j = 0; j < sortedData[i].degree; j++)
            edgeListGpu[tempIndex + j] = edgeList[nodePointersI[sortedData[i].index] + j];
        tempIndex += sortedData[i].degree;
    }
    std::vector<uint8_t> labelv(n, 0);
    bool *labelD = reinterpret_cast<bool *>(labelv.data());
    for (uint32_t i = 0; i < n; i++) value[i] = UINT_MAX;
    labelD[src] = true;
    value[src] = 1;
    std::vector<uint32_t> edgeListOverload(std::max<uint64_t>(1, m));
    std::vector<uint32_t> activeNodeListD(n), labeling(n), prefix(n), overloadDegree(n),
        overloadPrefix(n);
    launch([&] { setLabeling(n, labelD, labeling.data()); });
    uint32_t activeNodesNum = reduce_u32(labeling.data(), n);
    uint32_t iter = 0;
    while (activeNodesNum > 0) {
        iter++;
        exclusive_scan_u32(labeling.data(), n, prefix.data());
        launch([&] {
            setActiveNodeArrayAndNodePointerBySortOpt(n, activeNodeListD.data(), overloadDegree.data(),
                                                      labelD, prefix.data(), isInList, degree.data());
        });
        uint32_t overloadEdgeNum = reduce_u32(overloadDegree.data(), activeNodesNum);
        exclusive_scan_u32(overloadDegree.data(), activeNodesNum, overloadPrefix.data());
        if (overloadEdgeNum > 0) {
            for (uint32_t i = 0; i < activeNodesNum; i++) {  // main.cu:2353-2362
                uint32_t v = activeNodeListD[i];
                if (!isInList[v]) {
                    uint32_t dest = overloadPrefix[i], s = nodePointersI[v];
                    for (uint32_t j = 0; j < degree[v]; j++) edgeListOverload[dest + j] = edgeList[s + j];
                }
            }
        }
        launch([&] { setLabelDefault(activeNodesNum, activeNodeListD.data(), labelD); });
        launch([&] {
            bfs_kernelOptOfSorted(activeNodesNum, activeNodeListD.data(), ptrOfEdgeListGpu.data(),
                                  degree.data(), edgeListGpu.data(), edgeListOverload.data(), value,
                                  labelD, isInList, overloadPrefix.data());
        });
        launch([&] { setLabeling(n, labelD, labeling.data()); });
        activeNodesNum = reduce_u32(labeling.data(), n);
    }
    *iters_out = iter;
    return 0;
}

}  // namespace

extern "C" {

// variant: 0 bfsShare, 1 bfsOpt, 2 bfsAsync, 3 bfsAsyncSwap, 4 caculateInCommon
// (source 0), 5 caculateInShareOpt (source chosen by the reference, returned
// in *src_inout), 6 caculateInOptChooseByDegree, 10 ssspShare, 11 ssspOpt,
// 20 ccShare, 21 ccOpt.
// off_n has n entries (reference form); weight may be NULL for unweighted
// variants; budget_edges plays the role of max_partition_size.
int ref_run(int variant, uint32_t n, uint32_t m, const uint32_t *off_n, const uint32_t *col,
            const uint32_t *weight, uint32_t *src_inout, uint64_t budget_edges,
            uint32_t fragment_size, uint32_t *value, uint32_t *iters) {
    if (n == 0) return -1;
    Csr c = make_csr(n, m, off_n);
    std::vector<uint32_t> edges(col, col + m);
    edges.push_back(0);
    std::vector<EdgeWithWeight> wedges;
    if (weight) {
        wedges.resize(m + 1);
        for (uint32_t i = 0; i < m; i++) wedges[i] = EdgeWithWeight{col[i], weight[i]};
    }
    uint32_t src = *src_inout;
    switch (variant) {
        case 0: return run_share(0, c, edges.data(), nullptr, src, value, iters);
        case 1: return run_opt<uint32_t>(0, c, edges.data(), budget_edges, src, value, iters);
        case 2: return run_bfs_async(c, edges.data(), budget_edges, src, value, iters);
        case 3:
            return run_bfs_async_swap(c, edges.data(), budget_edges, fragment_size ? fragment_size : 4096,
                                      src, value, iters);
        case 4: *src_inout = 0; return run_share(0, c, edges.data(), nullptr, 0, value, iters);
        case 5: return run_bfs_share_opt(c, edges.data(), budget_edges, value, src_inout, iters);
        case 6: return run_bfs_by_degree(c, edges.data(), budget_edges, src, value, iters);
        case 10:
            if (!weight) return -1;
            return run_share(1, c, nullptr, wedges.data(), src, value, iters);
        case 11:
            if (!weight) return -1;
            return run_opt<EdgeWithWeight>(1, c, wedges.data(), budget_edges, src, value, iters);
        case 20: return run_share(2, c, edges.data(), nullptr, 0, value, iters);
        case 21: return run_opt<uint32_t>(2, c, edges.data(), budget_edges, 0, value, iters);
        default: return -1;
    }
}

}  // extern "C"
