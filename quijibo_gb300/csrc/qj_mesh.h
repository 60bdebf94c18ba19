// Host-side launchers of the marching-cubes pipeline (mesh.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>

#include "qj_params.h"

namespace qj {

// Scratch of one z-slab: cube flags per window layer, edge masks and vertex
// ids per window plane, the edge list of the slab's vertices, scan blocks.
struct MeshWindow {
  int X = 0, Y = 0;
  uint8_t* flags = nullptr;
  uint8_t* masks = nullptr;
  int32_t* vbase = nullptr;
  uint32_t* list = nullptr;
  long long* bsum = nullptr;
};

long long mesh_scan_blocks(long long n);

cudaError_t mesh_flags(const double* src, int X, int Y, long long n_layers, uint8_t* flags,
                       cudaStream_t s);
cudaError_t mesh_vertex_ids(MeshWindow& w, int j0, int j1, int lay_lo, int lay_hi,
                            long long running, long long* n_new, cudaStream_t s,
                            const std::function<cudaError_t(long long)>& ensure_list);
// Scratch of the FP32-first bisection with parked FP64 evaluations: one
// edge state per vertex of the mesh (mesh_edge_state_bytes() each, indexed
// by global vertex id), two parking lists of global vertex ids (list 0
// collects every slab's parked edges), two counters (zeroed once per mesh).
struct EdgeScratch {
  void* state;
  uint32_t* list[3];  // two parking lists (rounds alternate) and the FP64 sub-list
  unsigned long long* count;  // their three lengths
};
size_t mesh_edge_state_bytes();
// Vertex placement.  With hybrid bisection and a scratch, the edges that
// need FP64 values are parked and their vertices written by
// mesh_parked_finish after the last slab.
cudaError_t mesh_vertices(const MapParams& m, const GridParams& g, const IterParams& it,
                          int edge_mode, bool pow_ref, bool hybrid, const MeshWindow& w,
                          long long n, long long id0, int c0, const double* src, double* verts,
                          double iso, DevStats* st, const EdgeScratch* scratch, cudaStream_t s);
// Resolves every parked edge: rounds of one batched FP64 evaluation per
// parked edge and a resumption (host reads of the list sizes in between).
cudaError_t mesh_parked_finish(const MapParams& m, const GridParams& g, const IterParams& it,
                               bool pow_ref, double* verts, double iso, DevStats* st,
                               const EdgeScratch& sc, cudaStream_t s);
cudaError_t mesh_triangles(MeshWindow& w, int j0, int j1, long long running, int32_t* tris,
                           long long cap, long long* n_new, cudaStream_t s);
cudaError_t mesh_filter(const int32_t* tris, long long n, const double* verts, int32_t* out,
                        long long* bsum, long long* n_keep, cudaStream_t s);
cudaError_t mesh_to_float(const double* a, float* b, long long n, cudaStream_t s);

}  // namespace qj
