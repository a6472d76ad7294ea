// geom.cuh -- bounding box and derived Barnes-Hut constants (geom.cu).
#pragma once

#include "common.cuh"

namespace nbgb {

struct BBox {
  float min[3];
  float max[3];
  float inv[3];     // Morton normalisation 1 / (max - min + 0.001f)
  float center[3];  // Barnes-Hut root centre
  float half;       // Barnes-Hut root half size
  int valid;        // all bounds finite
};

int bbox_blocks(int64_t n);  // partials needs bbox_blocks(n) * 6 floats
void launch_bbox(const float4* pm, int64_t n, float* partials, BBox* box, uint32_t* err,
                 cudaStream_t st);

}  // namespace nbgb
