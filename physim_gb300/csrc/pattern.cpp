// pattern.cpp -- Hessian block pattern, scatter map and SELL layout, built on the host.
//
// The stored pattern is the one AMatrixSd builds on its first (triplet) assembly
// (source/PhySim/BasicTypes.cpp:64-78, 118-145; DerivativeAssembler.cpp:205-300):
// every tet contributes, for each local node pair (i, j <= i), a 3x3 block at
// (max(node_i, node_j), min(node_i, node_j)); node diagonal blocks are stored in
// full, duplicates are summed and structural zeros kept.  Expanded per DoF that
// is Eigen's lower CSC; per node it is a block-lower pattern with one block per
// node and one per mesh edge.  Block k is numbered column-major (C, then R),
// which is the order Eigen stores them in.
//
// For the device, the symmetric matrix is stored in full (V + 2E blocks) in
// SELL-32 order so a warp reads 32 rows' entries with one coalesced access, and
// the scatter map is inverted into per-block contribution lists ("segments")
// in element order, so the device sums each entry in exactly the order the
// reference's serial assembly does, without atomics.
#include "pattern.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace phx {

const int kPairI[10] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3};
const int kPairJ[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};

namespace {

inline double det3(const double* F) {
  return F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
         F[6] * (F[1] * F[5] - F[4] * F[2]);
}

// inverse of a column-major 3x3 (adjugate / det)
inline void inv3(const double* A, double d, double* Ai) {
  auto a = [&](int i, int j) { return A[i + 3 * j]; };
  double C[9];
  C[0] = a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1);
  C[1] = a(0, 2) * a(2, 1) - a(0, 1) * a(2, 2);
  C[2] = a(0, 1) * a(1, 2) - a(0, 2) * a(1, 1);
  C[3] = a(1, 2) * a(2, 0) - a(1, 0) * a(2, 2);
  C[4] = a(0, 0) * a(2, 2) - a(0, 2) * a(2, 0);
  C[5] = a(0, 2) * a(1, 0) - a(0, 0) * a(1, 2);
  C[6] = a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0);
  C[7] = a(0, 1) * a(2, 0) - a(0, 0) * a(2, 1);
  C[8] = a(0, 0) * a(1, 1) - a(0, 1) * a(1, 0);
  // C is the cofactor matrix stored column-major as C(i,j) = C[i + 3j] with the index
  // pattern above giving cofactor(i, j); inverse(i, j) = cofactor(j, i) / det.
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ai[i + 3 * j] = C[j + 3 * i] / d;
}

}  // namespace

void rebuild_load(const MeshIn& in, HostPattern& hp) {
  hp.hlin.assign(4 * (size_t)hp.n, 0.0);
  for (int v = 0; v < hp.n; ++v)
    for (int c = 0; c < 3; ++c) {
      double f = in.force ? in.force[3 * (size_t)v + c] : 0.0;
      hp.hlin[4 * (size_t)v + c] = f - hp.mass[v] * in.gravity[c];
    }
}

// BC_FixDoF in soft mode (BC_FixDoF.cpp:51-66): one EnergyElement_SoftConstraint per node
// with a nonzero stiffness, its target the given position or the node's rest position (the
// value the condition reads when it is built).
bool build_soft(const MeshIn& in, HostPattern& hp, std::string& err) {
  hp.soft.clear();
  if (!in.soft_k) return true;
  bool any = false;
  for (int v = 0; v < in.n; ++v) {
    const double k = in.soft_k[v];
    if (!(k >= 0.0) || !std::isfinite(k)) {
      err = "mesh: soft_k must be finite and >= 0";
      return false;
    }
    any = any || k > 0.0;
  }
  if (!any) return true;
  hp.soft.assign(4 * (size_t)in.n, 0.0);
  for (int v = 0; v < in.n; ++v) {
    const double* t = in.soft_target ? in.soft_target + 3 * (size_t)v : in.X0 + 3 * (size_t)v;
    for (int c = 0; c < 3; ++c) hp.soft[4 * (size_t)v + c] = t[c];
    hp.soft[4 * (size_t)v + 3] = in.soft_k[v];
  }
  return true;
}

bool build_pattern(const MeshIn& in, HostPattern& hp, std::string& err) {
  const int n = in.n, m = in.m;
  if (n <= 0 || m <= 0 || !in.X0 || !in.T || !in.lame || !in.rho) {
    err = "mesh: empty or missing arrays";
    return false;
  }
  if (!build_soft(in, hp, err)) return false;
  if ((int64_t)m * 10 > 2000000000LL) {
    err = "mesh: too many tets for 32-bit scatter indices";
    return false;
  }
  hp.n = n;
  hp.m = m;
  hp.tets.assign(in.T, in.T + 4 * (size_t)m);
  hp.model.assign(m, 0);
  if (in.model)
    for (int e = 0; e < m; ++e) {
      if (in.model[e] > 1) { err = "mesh: unknown material model"; return false; }
      hp.model[e] = in.model[e];
    }
  std::vector<char> used(n, 0);
  hp.rest64.resize(12 * (size_t)m);
  hp.rest32.resize(12 * (size_t)m);
  hp.mass.assign(n, 0.0);
  for (int e = 0; e < m; ++e) {
    const int32_t* t = &hp.tets[4 * (size_t)e];
    for (int a = 0; a < 4; ++a) {
      if (t[a] < 0 || t[a] >= n) { err = "mesh: node id out of range in tet " + std::to_string(e); return false; }
      for (int b = 0; b < a; ++b)
        if (t[a] == t[b]) { err = "mesh: repeated node in tet " + std::to_string(e); return false; }
      used[t[a]] = 1;
    }
    double Dm[9];
    for (int c = 0; c < 3; ++c)
      for (int r = 0; r < 3; ++r) Dm[r + 3 * c] = in.X0[3 * (size_t)t[c + 1] + r] - in.X0[3 * (size_t)t[0] + r];
    double d = det3(Dm);
    if (!(d > 0.0) || !std::isfinite(d)) {
      err = "mesh: non-positive rest volume in tet " + std::to_string(e);
      return false;
    }
    double lam = in.lame[2 * (size_t)e], mu = in.lame[2 * (size_t)e + 1], rho = in.rho[e];
    if (!std::isfinite(lam) || !std::isfinite(mu) || !std::isfinite(rho)) {
      err = "mesh: non-finite material parameter in tet " + std::to_string(e);
      return false;
    }
    double* R = &hp.rest64[12 * (size_t)e];
    inv3(Dm, d, R);
    R[9] = d / 6.0;  // quadrature weight (1/6) * det J (EnergyElement_FEM.cpp:87-91)
    R[10] = lam;
    R[11] = mu;
    for (int k = 0; k < 12; ++k) hp.rest32[12 * (size_t)e + k] = (float)R[k];
    // MassElement_Lumped::ComputeAndStore_Mass: rho * V / 4 per node
    double me = rho * (d / 6.0) / 4.0;
    for (int a = 0; a < 4; ++a) hp.mass[t[a]] += me;
  }
  for (int v = 0; v < n; ++v)
    if (!used[v]) { err = "mesh: node " + std::to_string(v) + " belongs to no tet"; return false; }

  // ---- lower blocks, column-major (C, R), and the scatter map ---------------
  // The tet pairs grouped by column C = min(node_i, node_j) (a counting sort); then per
  // column its distinct rows R in ascending order (a stamp per row and a sort of the few
  // distinct ones) and each pair's block index.
  // (each tet's four node ids are loaded once and its ten pairs unrolled)
  std::vector<int32_t> cnt(n + 1, 0);
  const int32_t* tt = hp.tets.data();
  for (int e = 0; e < m; ++e) {
    int32_t t[4];
    for (int a = 0; a < 4; ++a) t[a] = tt[4 * (size_t)e + a];
#pragma GCC unroll 10
    for (int p = 0; p < 10; ++p) cnt[std::min(t[kPairI[p]], t[kPairJ[p]]) + 1]++;
  }
  for (int v = 0; v < n; ++v) cnt[v + 1] += cnt[v];
  std::vector<int32_t> rows(cnt[n]), pairs(cnt[n]);  // row R and pair id 10 e + p, by column
  {
    std::vector<int32_t> pos(cnt.begin(), cnt.end() - 1);
    for (int e = 0; e < m; ++e) {
      int32_t t[4];
      for (int a = 0; a < 4; ++a) t[a] = tt[4 * (size_t)e + a];
#pragma GCC unroll 10
      for (int p = 0; p < 10; ++p) {
        const int32_t ni = t[kPairI[p]], nj = t[kPairJ[p]];
        const int q = pos[std::min(ni, nj)]++;
        rows[q] = std::max(ni, nj);
        pairs[q] = 10 * e + p;
      }
    }
  }
  // The scatter map's inverse (segments: each block's pairs in ascending pair id) comes out of
  // the same pass: a column's pairs are in ascending pair id, and its blocks are consecutive.
  hp.lo_colptr.assign(n + 1, 0);
  hp.scatter.resize(10 * (size_t)m);
  hp.seg_c.resize(10 * (size_t)m);
  hp.seg_ptr.assign(1, 0);
  hp.seg_ptr.reserve(cnt[n] / 3 + 2);
  std::vector<int32_t> lo_R;
  lo_R.reserve(cnt[n] / 3);
  std::vector<int32_t> seen(n, -1), block_of(n, 0), uniq, segpos;
  uniq.reserve(64);
  segpos.reserve(64);
  for (int C = 0; C < n; ++C) {
    uniq.clear();
    for (int q = cnt[C]; q < cnt[C + 1]; ++q)
      if (seen[rows[q]] != C) {
        seen[rows[q]] = C;
        uniq.push_back(rows[q]);
      }
    // a column has a few distinct rows (about 8-15): insertion sort
    for (size_t a = 1; a < uniq.size(); ++a) {
      const int32_t key = uniq[a];
      size_t b = a;
      for (; b > 0 && uniq[b - 1] > key; --b) uniq[b] = uniq[b - 1];
      uniq[b] = key;
    }
    const int32_t base = (int32_t)lo_R.size();
    for (size_t j = 0; j < uniq.size(); ++j) {
      lo_R.push_back(uniq[j]);
      block_of[uniq[j]] = base + (int32_t)j;
    }
    segpos.assign(uniq.size() + 1, 0);
    for (int q = cnt[C]; q < cnt[C + 1]; ++q) {
      const int32_t k = block_of[rows[q]];
      hp.scatter[pairs[q]] = k;
      segpos[k - base + 1]++;
    }
    segpos[0] = cnt[C];
    for (size_t j = 0; j < uniq.size(); ++j) {
      segpos[j + 1] += segpos[j];
      hp.seg_ptr.push_back(segpos[j + 1]);
    }
    for (int q = cnt[C]; q < cnt[C + 1]; ++q) hp.seg_c[segpos[block_of[rows[q]] - base]++] = pairs[q];
    hp.lo_colptr[C + 1] = (int32_t)lo_R.size();
  }
  hp.nlo = (int32_t)lo_R.size();
  hp.lo_rc.resize(2 * (size_t)hp.nlo);
  for (int C = 0; C < n; ++C)
    for (int k = hp.lo_colptr[C]; k < hp.lo_colptr[C + 1]; ++k) {
      hp.lo_rc[2 * (size_t)k] = lo_R[k];
      hp.lo_rc[2 * (size_t)k + 1] = C;
    }
  // every node has its diagonal block first in its column
  for (int C = 0; C < n; ++C)
    if (hp.lo_colptr[C + 1] == hp.lo_colptr[C] || lo_R[hp.lo_colptr[C]] != C) {
      err = "pattern: missing diagonal block";
      return false;
    }

  // ---- the node segments (each node's tet corners, in element order) -----
  hp.nseg_ptr.assign(n + 1, 0);
  for (size_t c = 0; c < 4 * (size_t)m; ++c) hp.nseg_ptr[hp.tets[c] + 1]++;
  for (int v = 0; v < n; ++v) hp.nseg_ptr[v + 1] += hp.nseg_ptr[v];
  hp.nseg_c.resize(4 * (size_t)m);
  {
    std::vector<int32_t> pos(hp.nseg_ptr.begin(), hp.nseg_ptr.end() - 1);
    for (size_t c = 0; c < 4 * (size_t)m; ++c) hp.nseg_c[pos[hp.tets[c]]++] = (int32_t)c;
  }

  // ---- full rows and SELL-32 slots ---------------------------------------
  // row v: [C < v from lower blocks (v, C)] [v] [R > v from column v]
  std::vector<int32_t> rowL_cnt(n + 1, 0);
  for (int k = 0; k < hp.nlo; ++k) {
    int R = hp.lo_rc[2 * (size_t)k], C = hp.lo_rc[2 * (size_t)k + 1];
    if (R != C) rowL_cnt[R + 1]++;
  }
  std::vector<int32_t> rowL_ptr(n + 1, 0);
  for (int v = 0; v < n; ++v) rowL_ptr[v + 1] = rowL_ptr[v] + rowL_cnt[v + 1];
  std::vector<int32_t> rowL_col(rowL_ptr[n]);
  hp.lo_slot.assign(hp.nlo, -1);
  hp.up_slot.assign(hp.nlo, -1);
  std::vector<int32_t> rowL_k(rowL_ptr[n]);
  {
    std::vector<int32_t> pos(rowL_ptr.begin(), rowL_ptr.end() - 1);
    for (int k = 0; k < hp.nlo; ++k) {  // k ascends with C, so each row list comes out sorted
      int R = hp.lo_rc[2 * (size_t)k], C = hp.lo_rc[2 * (size_t)k + 1];
      if (R != C) {
        rowL_col[pos[R]] = C;
        rowL_k[pos[R]] = k;
        pos[R]++;
      }
    }
  }
  hp.nchunks = (n + kChunk - 1) / kChunk;
  hp.chunk_off.assign(hp.nchunks + 1, 0);
  std::vector<int32_t> rowlen(n);
  for (int v = 0; v < n; ++v)
    rowlen[v] = (rowL_ptr[v + 1] - rowL_ptr[v]) + (hp.lo_colptr[v + 1] - hp.lo_colptr[v]);
  for (int c = 0; c < hp.nchunks; ++c) {
    int len = 0;
    for (int v = c * kChunk; v < std::min(n, (c + 1) * kChunk); ++v) len = std::max(len, rowlen[v]);
    hp.chunk_off[c + 1] = hp.chunk_off[c] + len * kChunk;
  }
  hp.nslots = hp.chunk_off[hp.nchunks];
  hp.slot_col.assign(hp.nslots, 0);
  hp.diag_slot.assign(n, -1);
  for (int c = 0; c < hp.nchunks; ++c) {
    int len = (hp.chunk_off[c + 1] - hp.chunk_off[c]) / kChunk;
    for (int lane = 0; lane < kChunk; ++lane) {
      int v = c * kChunk + lane;
      for (int k = 0; k < len; ++k) {
        int64_t s = hp.chunk_off[c] + (int64_t)k * kChunk + lane;
        hp.slot_col[s] = v < n ? v : 0;  // padding points at the row itself, value 0
      }
      if (v >= n) continue;
      int k = 0;
      for (int q = rowL_ptr[v]; q < rowL_ptr[v + 1]; ++q, ++k) {
        int64_t s = hp.chunk_off[c] + (int64_t)k * kChunk + lane;
        hp.slot_col[s] = rowL_col[q];
        hp.lo_slot[rowL_k[q]] = (int32_t)s;
      }
      for (int kk = hp.lo_colptr[v]; kk < hp.lo_colptr[v + 1]; ++kk, ++k) {
        int64_t s = hp.chunk_off[c] + (int64_t)k * kChunk + lane;
        int R = hp.lo_rc[2 * (size_t)kk];
        hp.slot_col[s] = R;
        if (R == v) {
          hp.diag_slot[v] = (int32_t)s;
          hp.lo_slot[kk] = (int32_t)s;
        } else {
          hp.up_slot[kk] = (int32_t)s;
        }
      }
    }
  }
  if (hp.nslots >= (int64_t)2000000000) {
    err = "pattern: too many blocks for 32-bit slot ids";
    return false;
  }
  // ---- per-tile node lists (shared-memory staging of the element stages) ---
  // Each tile of kTile consecutive tets lists its distinct nodes in ascending order (at most
  // 4 kTile, so a corner's index fits 16 bits); the element kernels load these once per tile.
  {
    const int nt = (m + kTile - 1) / kTile;
    hp.tile_nptr.assign(nt + 1, 0);
    hp.tile_nodes.clear();
    hp.tile_nodes.reserve((size_t)m);
    hp.tet_loc.resize(4 * (size_t)m);
    std::vector<int32_t> loc(n, -1), ids;
    ids.reserve(4 * kTile);
    for (int t = 0; t < nt; ++t) {
      const int e0 = t * kTile, e1 = std::min(m, e0 + kTile);
      ids.clear();
      for (size_t q = 4 * (size_t)e0; q < 4 * (size_t)e1; ++q)
        if (loc[hp.tets[q]] < 0) {
          loc[hp.tets[q]] = 0;
          ids.push_back(hp.tets[q]);
        }
      std::sort(ids.begin(), ids.end());
      for (size_t k = 0; k < ids.size(); ++k) loc[ids[k]] = (int32_t)k;
      for (size_t q = 4 * (size_t)e0; q < 4 * (size_t)e1; ++q) hp.tet_loc[q] = (uint16_t)loc[hp.tets[q]];
      for (int32_t v : ids) loc[v] = -1;
      hp.tile_nodes.insert(hp.tile_nodes.end(), ids.begin(), ids.end());
      hp.tile_nptr[t + 1] = (int32_t)hp.tile_nodes.size();
    }
  }
  // ---- boundary conditions ------------------------------------------------
  hp.fixmask.assign(n, 0);
  if (in.fixed)
    for (int v = 0; v < n; ++v)
      for (int c = 0; c < 3; ++c)
        if (in.fixed[3 * (size_t)v + c]) hp.fixmask[v] |= (uint8_t)(1u << c);
  rebuild_load(in, hp);
  return true;
}

BaseLayout base_layout(const HostPattern& hp) {
  BaseLayout L;
  size_t off = 0;
  auto part = [&](BaseLayout::Part& p, size_t count, size_t elem) {
    p.off = off;
    p.bytes = std::max<size_t>(count, 1) * elem;
    off += (p.bytes + 255) & ~(size_t)255;
  };
  const size_t n4 = 4 * (size_t)hp.n, m = hp.m;
  part(L.tets, hp.tets.size(), 4);
  part(L.rest64, hp.rest64.size(), 8);
  part(L.rest32, hp.rest32.size(), 4);
  part(L.tile_nptr, hp.tile_nptr.size(), 4);
  part(L.tile_nodes, hp.tile_nodes.size(), 4);
  part(L.tet_loc, hp.tet_loc.size(), 2);
  part(L.model, hp.model.size(), 1);
  part(L.chunk_off, hp.chunk_off.size(), 4);
  part(L.slot_col, hp.slot_col.size(), 4);
  part(L.diag_slot, hp.diag_slot.size(), 4);
  part(L.lo_rc, hp.lo_rc.size(), 4);
  part(L.lo_slot, hp.lo_slot.size(), 4);
  part(L.up_slot, hp.up_slot.size(), 4);
  part(L.seg_ptr, hp.seg_ptr.size(), 4);
  part(L.seg_c, hp.seg_c.size(), 4);
  part(L.nseg_ptr, hp.nseg_ptr.size(), 4);
  part(L.nseg_c, hp.nseg_c.size(), 4);
  part(L.fixmask, hp.fixmask.size(), 1);
  part(L.mass, hp.mass.size(), 8);
  part(L.hlin, hp.hlin.size(), 8);
  if (!hp.soft.empty()) part(L.soft, hp.soft.size(), 8);
  part(L.x, n4, 8);
  part(L.xrest, n4, 8);
  L.upload_end = off;
  for (auto& v : L.vec) part(v, n4, 8);
  part(L.counter, 1, 4);
  part(L.log, 4 * (size_t)kLogCap, 8);
  part(L.st, 1, sizeof(NState));
  part(L.opts, 1, sizeof(DevOpts));
  L.zero_end = off;
  auto tiles = [](int count) { return (size_t)((count + kTile - 1) / kTile); };
  const size_t maxt = std::max({tiles(hp.m), (size_t)hp.nchunks, tiles(hp.nlo)});
  part(L.eloc, m, 8);
  part(L.gloc, 12 * m, 8);
  part(L.partials, maxt * kPartials, 8);
  L.total = off;
  return L;
}

// The uploaded part of the base block, [0, upload_end), written into dst.
void pack_base(const HostPattern& hp, const double* X0, const BaseLayout& L, char* dst) {
  auto put = [&](const BaseLayout::Part& p, const void* src, size_t bytes) {
    if (bytes) std::memcpy(dst + p.off, src, bytes);
  };
  put(L.tets, hp.tets.data(), hp.tets.size() * 4);
  put(L.rest64, hp.rest64.data(), hp.rest64.size() * 8);
  put(L.rest32, hp.rest32.data(), hp.rest32.size() * 4);
  put(L.tile_nptr, hp.tile_nptr.data(), hp.tile_nptr.size() * 4);
  put(L.tile_nodes, hp.tile_nodes.data(), hp.tile_nodes.size() * 4);
  put(L.tet_loc, hp.tet_loc.data(), hp.tet_loc.size() * 2);
  put(L.model, hp.model.data(), hp.model.size());
  put(L.chunk_off, hp.chunk_off.data(), hp.chunk_off.size() * 4);
  put(L.slot_col, hp.slot_col.data(), hp.slot_col.size() * 4);
  put(L.diag_slot, hp.diag_slot.data(), hp.diag_slot.size() * 4);
  put(L.lo_rc, hp.lo_rc.data(), hp.lo_rc.size() * 4);
  put(L.lo_slot, hp.lo_slot.data(), hp.lo_slot.size() * 4);
  put(L.up_slot, hp.up_slot.data(), hp.up_slot.size() * 4);
  put(L.seg_ptr, hp.seg_ptr.data(), hp.seg_ptr.size() * 4);
  put(L.seg_c, hp.seg_c.data(), hp.seg_c.size() * 4);
  put(L.nseg_ptr, hp.nseg_ptr.data(), hp.nseg_ptr.size() * 4);
  put(L.nseg_c, hp.nseg_c.data(), hp.nseg_c.size() * 4);
  put(L.fixmask, hp.fixmask.data(), hp.fixmask.size());
  put(L.mass, hp.mass.data(), hp.mass.size() * 8);
  put(L.hlin, hp.hlin.data(), hp.hlin.size() * 8);
  if (!hp.soft.empty()) put(L.soft, hp.soft.data(), hp.soft.size() * 8);
  double* x = reinterpret_cast<double*>(dst + L.x.off);
  for (int v = 0; v < hp.n; ++v) {
    for (int c = 0; c < 3; ++c) x[4 * (size_t)v + c] = X0[3 * (size_t)v + c];
    x[4 * (size_t)v + 3] = 0.0;
  }
  std::memcpy(dst + L.xrest.off, x, 4 * (size_t)hp.n * sizeof(double));
}

}  // namespace phx
