// Host-side internals shared by the translation units: handle structs, error
// reporting, allocation helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "common.cuh"
#include "guard.h"

struct rmg_map {
  int device;
  uint32_t n_vertices;
  uint32_t n_faces;
  uint32_t n_nodes;
  uint32_t depth;
  float lo[3], hi[3];
  // device arrays
  float* d_vertices;          // 3*n_vertices
  uint32_t* d_faces;          // 3*n_faces
  rmg::Node* d_nodes;         // n_nodes
  rmg::Tri* d_tris;           // n_faces (leaf order)
  uint32_t* d_leaf_order;     // n_faces: face id of each leaf
  int* d_leaf_parent;         // n_faces: parent node of each leaf
  unsigned int* d_flags;      // n_nodes refit visit counters
  unsigned int* d_status;     // 1 word: device error status
  // 4-wide tree collapsed from the binary one (wide.cu)
  rmg::Node4* d_nodes4;       // n_nodes4
  int* d_src4;                // 4*n_nodes4: binary record (2*parent + side) of each slot, -1 empty
  uint32_t n_nodes4;
  uint32_t depth4;            // levels of the wide tree
  // 8-wide tree with quantized boxes (wide8.cu)
  rmg::Node8* d_nodes8;       // n_nodes8
  int* d_src8;                // 8*n_nodes8: binary record of each slot, -1 empty
  rmg::Tri* d_tris8;          // n_faces: the triangles in 8-wide leaf order
  int* d_tri8_src;            // n_faces: packed triangle of each d_tris8 entry
  uint32_t n_nodes8;
  uint32_t depth8;            // levels of the 8-wide tree
};

struct rmg_sensor {
  int device;
  rmg_model model;            // copy; dirs/origs pointers cleared
  uint32_t width, height;
  float* d_dirs;              // 3*width*height
  float* d_origs;             // 3*width*height (OnDn only)
  uint32_t* d_order;          // width*height visiting order (O1Dn / OnDn tables sorted for coherence), or NULL
};

namespace rmg {

void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
// Maps a CUDA error to a status, recording the message.  Returns RMG_OK for
// cudaSuccess.
int cuda_status(cudaError_t e, const char* what);

#define RMG_CUDA_TRY(expr)                                     \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) return ::rmg::cuda_status(_e, #expr); \
  } while (0)

template <typename T>
int dev_alloc(T** p, size_t count, const char* what) {
  *p = nullptr;
  if (count == 0) return RMG_OK;
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? RMG_ERR_OOM : RMG_ERR_CUDA,
                std::string("cudaMalloc failed for ") + what);
  }
  return RMG_OK;
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

DeviceMap device_view(const rmg_map* m);
int wide_build(rmg_map* m, cudaStream_t st);
// Binned-SAH topology of a map's n >= 2 faces (csrc/sah.cu); synchronises.
int sah_build_topology(rmg_map* m, cudaStream_t st, uint32_t* d_order);
int wide_refit(rmg_map* m, cudaStream_t st);
void wide_free(rmg_map* m);
int wide8_build(rmg_map* m, cudaStream_t st);
int wide8_refit(rmg_map* m, cudaStream_t st);
void wide8_free(rmg_map* m);
SensorDev device_view(const rmg_sensor* s);

int device_sm_count();

}  // namespace rmg
