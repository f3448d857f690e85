// pattern.h -- host-side construction of the Hessian block pattern and the scatter map.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "phx_types.h"

namespace phx {

struct MeshIn {
  int32_t n = 0, m = 0;
  const double* X0 = nullptr;
  const int32_t* T = nullptr;
  const double* lame = nullptr;
  const double* rho = nullptr;
  const uint8_t* model = nullptr;
  const uint8_t* fixed = nullptr;
  const double* force = nullptr;
  double gravity[3] = {0, 0, 0};
  const double* soft_k = nullptr;       // [n] soft fixed-position stiffness per node (0: none), or null
  const double* soft_target = nullptr;  // [3n] its targets; null: X0
};

// Everything the device needs, built once per mesh on the host.
struct HostPattern {
  int32_t n = 0, m = 0, nlo = 0, nchunks = 0;
  int64_t nslots = 0;
  std::vector<int32_t> tets;          // [4m]
  std::vector<double> rest64;         // [12m]
  std::vector<float> rest32;          // [12m]
  std::vector<int32_t> tile_nptr;     // [tiles(m)+1] unique nodes of each 128-tet tile ...
  std::vector<int32_t> tile_nodes;    // ... ascending, concatenated
  std::vector<uint16_t> tet_loc;      // [4m] each corner's index in its tile's node list
  std::vector<uint8_t> model;         // [m]
  std::vector<int32_t> lo_rc;         // [2 nlo] (R, C), column-major block order (C, then R)
  std::vector<int32_t> lo_colptr;     // [n+1] lower blocks of block column C: [lo_colptr[C], lo_colptr[C+1])
  std::vector<int32_t> scatter;       // [10m] lower block of each (tet, local pair)
  std::vector<int32_t> seg_ptr;       // [nlo+1]
  std::vector<int32_t> seg_c;         // [10m]
  std::vector<int32_t> nseg_ptr;      // [n+1]
  std::vector<int32_t> nseg_c;        // [4m]
  std::vector<int32_t> chunk_off;     // [nchunks+1]
  std::vector<int32_t> slot_col;      // [nslots]
  std::vector<int32_t> diag_slot;     // [n]
  std::vector<int32_t> lo_slot;       // [nlo]
  std::vector<int32_t> up_slot;       // [nlo]
  std::vector<uint8_t> fixmask;       // [n]
  std::vector<double> mass;           // [n]
  std::vector<double> hlin;           // [4n]  f - m g
  std::vector<double> soft;           // [4n]  soft fixed position (target, k) per node; empty: none
};

// Validates the mesh and builds the pattern; returns false with a message on bad input.
bool build_pattern(const MeshIn& in, HostPattern& out, std::string& err);

// Recomputes hlin = f - m g after a load update.
void rebuild_load(const MeshIn& in, HostPattern& hp);

// Local node pairs (i, j <= i) in the reference's propagate order (DerivativeAssembler.cpp:205-245).
extern const int kPairI[10];
extern const int kPairJ[10];

// An instance's base block in the arena: the arrays uploaded from its host pattern (and its
// positions, twice: current and rest), then the arrays that start at zero, then per-element
// scratch, each at a 256-byte aligned offset.  One copy from pinned memory and one memset set
// it up.
struct BaseLayout {
  struct Part {
    size_t off = 0, bytes = 0;
  };
  Part tets, rest64, rest32, tile_nptr, tile_nodes, tet_loc, model, chunk_off, slot_col, diag_slot, lo_rc, lo_slot,
      up_slot, seg_ptr, seg_c, nseg_ptr, nseg_c, fixmask, mass, hlin, soft, x, xrest;
  size_t upload_end = 0;
  Part vec[11], counter, log, st, opts;  // vec: xs, dx, g, gn, dxprev, x0, v0, v, r64, bvec, xback
  size_t zero_end = 0;
  Part eloc, gloc, partials;
  size_t total = 0;
};

BaseLayout base_layout(const HostPattern& hp);
// The uploaded part of the base block, [0, upload_end), written into dst (X0: rest positions [3n]).
void pack_base(const HostPattern& hp, const double* X0, const BaseLayout& L, char* dst);

}  // namespace phx
