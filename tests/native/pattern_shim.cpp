// Test-only C shim over the product's host pattern builder (physim_gb300/csrc/pattern.cpp),
// so the pattern, scatter map and SELL layout can be checked on a machine without a GPU.
#include <cstring>
#include <string>

#include "pattern.h"

static phx::HostPattern g_hp;
static std::string g_err;

extern "C" {

int pat_build(int n, int m, const double* X0, const int* T, const double* lame, const double* rho,
              const unsigned char* model, const unsigned char* fixed, const double* force, const double* grav) {
  phx::MeshIn in;
  in.n = n; in.m = m; in.X0 = X0; in.T = T; in.lame = lame; in.rho = rho; in.model = model;
  in.fixed = fixed; in.force = force;
  for (int c = 0; c < 3; ++c) in.gravity[c] = grav[c];
  g_hp = phx::HostPattern();
  return phx::build_pattern(in, g_hp, g_err) ? 0 : -1;
}

// the same with BC_FixDoF soft-mode data (soft_k [n], soft_target [3n] or NULL)
int pat_build_soft(int n, int m, const double* X0, const int* T, const double* lame, const double* rho,
                   const unsigned char* model, const unsigned char* fixed, const double* force, const double* grav,
                   const double* soft_k, const double* soft_target) {
  phx::MeshIn in;
  in.n = n; in.m = m; in.X0 = X0; in.T = T; in.lame = lame; in.rho = rho; in.model = model;
  in.fixed = fixed; in.force = force;
  for (int c = 0; c < 3; ++c) in.gravity[c] = grav[c];
  in.soft_k = soft_k;
  in.soft_target = soft_target;
  g_hp = phx::HostPattern();
  return phx::build_pattern(in, g_hp, g_err) ? 0 : -1;
}

long long pat_soft_size() { return (long long)g_hp.soft.size(); }

const char* pat_error() { return g_err.c_str(); }

// sizes: n, m, nlo, nchunks, nslots
void pat_sizes(long long* out) {
  out[0] = g_hp.n; out[1] = g_hp.m; out[2] = g_hp.nlo; out[3] = g_hp.nchunks; out[4] = g_hp.nslots;
}

#define GET(name, type)                                                                    \
  void pat_##name(type* out) {                                                             \
    if (!g_hp.name.empty()) std::memcpy(out, g_hp.name.data(), g_hp.name.size() * sizeof(type)); \
  }
GET(lo_rc, int)
GET(lo_colptr, int)
GET(scatter, int)
GET(seg_ptr, int)
GET(seg_c, int)
GET(nseg_ptr, int)
GET(nseg_c, int)
GET(chunk_off, int)
GET(slot_col, int)
GET(diag_slot, int)
GET(lo_slot, int)
GET(up_slot, int)
GET(rest64, double)
GET(mass, double)
GET(hlin, double)
GET(fixmask, unsigned char)
GET(soft, double)

// The device base block of the last pattern: every part's (offset, bytes) in declaration order
// (23 uploaded parts, 11 zeroed vectors, counter, log, state, options, 3 scratch parts: 41), then
// upload_end, zero_end, total.  Returns the number of values written (85).
int pat_layout(long long* out) {
  const phx::BaseLayout L = phx::base_layout(g_hp);
  const phx::BaseLayout::Part* parts[] = {
      &L.tets, &L.rest64, &L.rest32, &L.tile_nptr, &L.tile_nodes, &L.tet_loc, &L.model, &L.chunk_off,
      &L.slot_col, &L.diag_slot, &L.lo_rc, &L.lo_slot, &L.up_slot, &L.seg_ptr, &L.seg_c, &L.nseg_ptr,
      &L.nseg_c, &L.fixmask, &L.mass, &L.hlin, &L.soft, &L.x, &L.xrest,
      &L.vec[0], &L.vec[1], &L.vec[2], &L.vec[3], &L.vec[4], &L.vec[5], &L.vec[6], &L.vec[7], &L.vec[8],
      &L.vec[9], &L.vec[10], &L.counter, &L.log, &L.st, &L.opts, &L.eloc, &L.gloc, &L.partials};
  int k = 0;
  for (auto* p : parts) {
    out[k++] = (long long)p->off;
    out[k++] = (long long)p->bytes;
  }
  out[k++] = (long long)L.upload_end;
  out[k++] = (long long)L.zero_end;
  out[k++] = (long long)L.total;
  return k;
}

// The packed upload of the last pattern (upload_end bytes) with rest positions X0.
void pat_pack(const double* X0, char* dst) { phx::pack_base(g_hp, X0, phx::base_layout(g_hp), dst); }
}
