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
}
