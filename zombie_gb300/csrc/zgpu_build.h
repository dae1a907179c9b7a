// zgpu_build.h -- host-side boundary preprocessing (adjacency, silhouette flags, BVH).
#pragma once

#include <string>
#include <vector>
#include <vector_types.h>
#include <vector_functions.h>

namespace zg {

struct HostBoundary {
    int dim = 2;
    int kind = 0;
    int nPrims = 0;
    int nNodes = 0;
    int depth = 0;
    int width = 4;                // children per node (8: 3D absorbing boundaries only)
    float signedVolume = 0.0f;
    std::vector<float4> nodes;    // nNodes * 2 * width
    std::vector<float4> cones;    // reflecting only: nNodes * 8 (per child cone, then per-child max Robin coeff)
    std::vector<float4> prims;    // nPrims * (1 | 3)
    std::vector<float4> sil;      // reflecting only: nPrims * (2 | 3)
    std::vector<int> primIndex;   // leaf slot -> caller's primitive index
    // silhouette-candidate tree (reflecting boundaries): one record per non-ignored vertex
    // (2D) / edge (3D), deduplicated; 2D record 2 float4, 3D record 4 float4
    int silNodes = 0;
    int silDepth = 0;
    int silFeatures = 0;
    std::vector<float4> silTree;    // silNodes * 8 (wide nodes, same layout as `nodes`)
    std::vector<float4> silCones;   // silNodes * 8 (child cones)
    std::vector<float4> silFeat;    // silFeatures * (2 | 4)
};

// kind: 0 absorbing, 1 Neumann, 2 Robin (include/zgpu.h).  Returns false with a message.
bool buildBoundary(int dim, const float* positions, int nVertices, const int* indices, int nPrims, int kind,
                   const float* minRobin, const float* maxRobin, bool solveDoubleSided, float silhouettePrecision,
                   HostBoundary& out, std::string& error, int width = 4);

}  // namespace zg
