// Host-side launchers of the marching-cubes pipeline (mesh.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>

#include "qj_params.h"

namespace qj {

// A cube with triangles, in scan order: its cell (y * X + x), its global
// plane with the case flag in the top byte, and the global index of its
// first triangle.
struct McCube {
  uint32_t r;
  uint32_t gzf;
  long long tb;
};

// Device-side counts of one slab's classification.
struct McTotals {
  long long nv, nc;  // vertices and cubes with triangles of the slab
  long long nt;      // triangles of the cubes of the last cube scan
  long long split;   // the slab's cube entries below its last cube layer
};

// The counts of a mesh run kept on the device, for the fixed launch
// sequence (qjg_mesh_stream_async): every launcher below that takes a run
// reads its counts and offsets from here instead of from host arguments, so
// no host read sits between the kernels.
struct McRun {
  long long nv;       // vertices of the slabs so far (first id of the slab's vertices)
  long long nt;       // triangles of the cube entries scanned so far
  long long n_carry;  // cube entries carried into the slab's list
  long long prev_nc;  // the previous slab's new cube entries
  long long n_new;    // the slab's vertices
  long long nc;       // the slab's new cube entries
  long long n_filter; // triangles the degenerate filter reads (0 after an overflow)
  long long keep;     // triangles kept by the degenerate filter
  long long cap_v, cap_list, cap_cubes, cap_t;  // capacities of the run's buffers
  int overflow;       // a count outgrew a capacity: nothing more is written
  int pad;
};

// Scratch of one z-slab.  Window planes j <-> global plane c0 - 1 + j: edge
// masks and vertex ids per window plane (plane c0 - 1 carried over from the
// previous slab); per classified plane the activity bits, sparse voxel codes
// and unit counts; the edge list of the slab's vertices; scan blocks.
struct MeshWindow {
  int X = 0, Y = 0;
  uint8_t* masks = nullptr;
  int32_t* vbase = nullptr;
  uint32_t* list = nullptr;
  long long* bsum = nullptr;  // 2 per scan block
  uint32_t* sign = nullptr;   // MESH_UNIT_WORDS per unit, every plane of the window
  uint32_t* bits = nullptr;   // MESH_UNIT_WORDS per unit
  uint32_t* ucount = nullptr;
  McTotals* tot = nullptr;
};

long long mesh_scan_blocks(long long n);
// classification units (row segments of one plane) of `planes` planes
long long mesh_units(int X, int Y, int planes);
// Words of activity bits per unit (64 voxels: even x, odd x).
constexpr int MESH_UNIT_WORDS = 2;

// Classify voxel planes [0, Pv) of src (P planes, global plane gz0 first;
// Pv = P - 1, or P on the grid's last plane): sign words of every plane,
// activity words and unit counts, their scan, the slab totals in w.tot (nv,
// nc).
cudaError_t mesh_classify(const MeshWindow& w, const double* src, int P, int Pv, int gz0,
                          cudaStream_t s);
// The slab's vertex ids, masks and edge list (window planes 1..Pv) and its
// cube entries (written from `cubes`); u_split = the first unit of the last
// cube layer (-1 on the last slab), whose entry offset goes to w.tot->split.
cudaError_t mesh_emit(const MeshWindow& w, const double* src, int P, int Pv, int gz0,
                      long long u_split, long long id0, McCube* cubes, cudaStream_t s);
// The first triangle of each of the nc cube entries (global index, from t0);
// their triangle count goes to w.tot->nt.
cudaError_t mesh_cube_scan(const MeshWindow& w, McCube* cubes, long long nc, long long t0,
                           cudaStream_t s);
// Triangles of cube entries [0, n_carry + split) (all on the last slab);
// unless last, the remaining entries move to the front of `next`.
cudaError_t mesh_triangles(const MeshWindow& w, const McCube* cubes, long long n_carry,
                           long long nc, bool last, int zbase, McCube* next, int32_t* tris,
                           long long cap, cudaStream_t s);
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
// Vertex placement (pow_mode as for launch_field64).  With hybrid bisection and a scratch, the edges that
// need FP64 values are parked and their vertices written by
// mesh_parked_finish after the last slab.
cudaError_t mesh_vertices(const MapParams& m, const GridParams& g, const IterParams& it,
                          int edge_mode, int pow_mode, bool hybrid, const MeshWindow& w,
                          long long n, long long id0, int c0, const double* src, double* verts,
                          double iso, DevStats* st, const EdgeScratch* scratch, cudaStream_t s);
// Resolves every parked edge: rounds of one batched FP64 evaluation per
// parked edge and a resumption (host reads of the list sizes in between).
cudaError_t mesh_parked_finish(const MapParams& m, const GridParams& g, const IterParams& it,
                               int pow_mode, double* verts, double iso, DevStats* st,
                               const EdgeScratch& sc, cudaStream_t s);
cudaError_t mesh_filter(const int32_t* tris, long long n, const double* verts, int32_t* out,
                        long long* bsum, long long* n_keep, cudaStream_t s);
cudaError_t mesh_to_float(const double* a, float* b, long long n, cudaStream_t s);

// ---- the same phases with the counts on the device (McRun) ----
// run <- zero counts and the capacities
cudaError_t mesh_run_init(McRun* run, long long cap_v, long long cap_list, long long cap_cubes,
                          long long cap_t, cudaStream_t s);
// after a slab's classification: its counts and carry from w.tot, the
// previous slab's triangles added, capacities checked (first: c0 == 0)
cudaError_t mesh_run_slab(McRun* run, const McTotals* tot, bool first, cudaStream_t s);
// after a slab's vertices: vertex base and previous cube count advance
cudaError_t mesh_run_next(McRun* run, cudaStream_t s);
// after the last slab: its triangles added, the triangle capacity checked
cudaError_t mesh_run_final(McRun* run, const McTotals* tot, bool any_slab, cudaStream_t s);
cudaError_t mesh_emit_run(const MeshWindow& w, const double* src, int P, int Pv, int gz0,
                          long long u_split, McCube* cubes, const McRun* run, cudaStream_t s);
cudaError_t mesh_cube_scan_run(const MeshWindow& w, McCube* cubes, McRun* run,
                               long long cap_cubes, cudaStream_t s);
cudaError_t mesh_vertices_run(const MapParams& m, const GridParams& g, const IterParams& it,
                              int edge_mode, int pow_mode, bool hybrid, const MeshWindow& w,
                              int c0, const double* src, double* verts, double iso, DevStats* st,
                              const EdgeScratch* scratch, const McRun* run, cudaStream_t s);
// the parked edges in a fixed number of rounds (8, the most any edge needs)
cudaError_t mesh_parked_finish_fixed(const MapParams& m, const GridParams& g,
                                     const IterParams& it, int pow_mode, double* verts,
                                     double iso, DevStats* st, const EdgeScratch& sc,
                                     cudaStream_t s);
cudaError_t mesh_triangles_run(const MeshWindow& w, const McCube* cubes, bool last, int zbase,
                               McCube* next, int32_t* tris, long long cap, const McRun* run,
                               cudaStream_t s);
// degenerate filter of run->nt triangles (at most cap_t) into out; run->keep
cudaError_t mesh_filter_run(const int32_t* tris, const double* verts, int32_t* out,
                            long long* bsum, McRun* run, long long cap_t, cudaStream_t s);
// the run's vertices (FP64 and/or FP32) and kept triangles to the caller's buffers
cudaError_t mesh_copy_out_run(const double* verts, double* v64, float* v32, const int32_t* kept,
                              int32_t* tris, const McRun* run, cudaStream_t s);
// acc += the field call's counters (every field counter but the tile position)
cudaError_t mesh_stats_add(DevStats* acc, const DevStats* st, cudaStream_t s);

}  // namespace qj
