// phx_oracle.cpp -- CPU restatement of PhySim's nonlinear tet-FEM Newton path.
//
// TEST INFRASTRUCTURE ONLY: the checker the GPU library is compared against,
// and the timed CPU baseline of the benchmark.  The product never links it.
//
// What is restated, and from where (paths relative to the reference project):
//   element kinematics  source/PhySim/Geometry/Polytopes/ShapeFunctions.cpp:89-158,
//                       include/PhySim/Geometry/Polytopes/ShapeFunctions.h:391-442,
//                       include/PhySim/Geometry/Polytopes/Quadratures.h:117-137
//   element E / g / H   source/PhySim/Physics/Elements/EnergyElement_FEM.cpp:59-222
//   material laws       include/PhySim/Physics/Elements/MaterialModels.h:166-299 (formulas
//                       derived here; pinned against the generated .mcg code by golden vectors)
//   lumped mass/gravity source/PhySim/Physics/Elements/MassElement_Lumped.cpp:47-76
//   nodal forces        source/PhySim/Physics/Elements/EnergyElement_Force.cpp:43-56
//   assembly + fixing   source/PhySim/Physics/Simulables/Simulable.cpp:321-760,
//                       source/PhySim/BasicTypes.cpp:18-164,
//                       source/PhySim/Utils/DerivativeAssembler.cpp:205-300
//   problems            source/PhySim/Solvers/OptimProblem_BasicStatic.cpp:42-121,
//                       source/PhySim/Solvers/OptimProblem_BasicDynamic.cpp:58-168
//   Newton + LS         source/PhySim/Solvers/OptimSolver.cpp:148-495, 688-736,
//                       source/PhySim/Solvers/OptimSolver_USQP_LS.cpp:18-68
//   linear solvers      source/PhySim/Solvers/LinearSolver.cpp:29-66,
//                       source/PhySim/Solvers/LinearSolver_EigenLDLT.cpp:49-154,
//                       source/PhySim/Solvers/LinearSolver_EigenCG.cpp:51-125
//
// The reference's linear algebra is Eigen (unpinned version): SimplicialLDLT
// and ConjugateGradient<SparseMatrix, Lower, DiagonalPreconditioner>.  Eigen is
// not available, so the LDL^T here is an own up-looking simplicial
// factorisation written from the published algorithm (T. A. Davis, "Algorithm
// 849: a concise sparse Cholesky factorization package", ACM TOMS 31(4), 2005)
// over an own geometric nested-dissection node ordering, and the CG is the
// textbook preconditioned CG with Eigen's documented stopping rule
// (||r|| < tol * ||b||, zero right-hand side gives x = 0).
#include "phx_oracle.h"

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using clk = std::chrono::steady_clock;
static double secs(clk::time_point a, clk::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

// ---------------------------------------------------------------------------
// 3x3 helpers, column-major storage F(i,j) = F[i + 3j] (MathUtils::Vectorize).
// ---------------------------------------------------------------------------
inline double det3(const double* F) {
  return F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
         F[6] * (F[1] * F[5] - F[4] * F[2]);
}
// cofactor matrix (MathUtils.h:64-74), column-major
inline void cofactor3(const double* F, double* C) {
  auto f = [&](int i, int j) { return F[i + 3 * j]; };
  C[0 + 3 * 0] = f(1, 1) * f(2, 2) - f(1, 2) * f(2, 1);
  C[1 + 3 * 0] = f(0, 2) * f(2, 1) - f(0, 1) * f(2, 2);
  C[2 + 3 * 0] = f(0, 1) * f(1, 2) - f(0, 2) * f(1, 1);
  C[0 + 3 * 1] = f(1, 2) * f(2, 0) - f(1, 0) * f(2, 2);
  C[1 + 3 * 1] = f(0, 0) * f(2, 2) - f(0, 2) * f(2, 0);
  C[2 + 3 * 1] = f(0, 2) * f(1, 0) - f(0, 0) * f(1, 2);
  C[0 + 3 * 2] = f(1, 0) * f(2, 1) - f(1, 1) * f(2, 0);
  C[1 + 3 * 2] = f(0, 1) * f(2, 0) - f(0, 0) * f(2, 1);
  C[2 + 3 * 2] = f(0, 0) * f(1, 1) - f(0, 1) * f(1, 0);
}

// ---------------------------------------------------------------------------
// Material laws.  psi(F), P = dpsi/dF and dP/dF with the vec convention of the
// reference: index a = i + 3j for entry (i,j), dPdF[a*9 + b] = dP_a / dF_b.
// ---------------------------------------------------------------------------
// Compressible Neo-Hookean (MaterialModels.h:235-299):
//   psi = mu/2 (tr(F^T F) - 3 - log J^2) + lambda/8 (log J^2)^2
//   P   = mu F + (lambda/2 log J^2 - mu) F^-T
//   dP_ij/dF_kl = mu d_ik d_jl + (mu - lambda/2 log J^2) G_il G_kj + lambda G_kl G_ij,  G = F^-T
void conh(double lam, double mu, const double* F, double* psi, double* P, double* D) {
  double J = det3(F);
  double logJ2 = std::log(J * J);
  if (psi) {
    double I1 = 0;
    for (int a = 0; a < 9; ++a) I1 += F[a] * F[a];
    *psi = mu * (I1 - 3.0 - logJ2) / 2.0 + lam * logJ2 * logJ2 / 8.0;
  }
  if (!P && !D) return;
  double G[9];
  cofactor3(F, G);
  for (int a = 0; a < 9; ++a) G[a] /= J;
  if (P) {
    double c = 0.5 * lam * logJ2 - mu;
    for (int a = 0; a < 9; ++a) P[a] = mu * F[a] + c * G[a];
  }
  if (D) {
    double c = mu - 0.5 * lam * logJ2;
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i)
        for (int l = 0; l < 3; ++l)
          for (int k = 0; k < 3; ++k) {
            double v = c * G[i + 3 * l] * G[k + 3 * j] + lam * G[k + 3 * l] * G[i + 3 * j];
            if (i == k && j == l) v += mu;
            D[(i + 3 * j) * 9 + (k + 3 * l)] = v;
          }
  }
}

// Saint-Venant Kirchhoff (MaterialModels.h:166-230):
//   E = (F^T F - I)/2, psi = lambda/2 tr(E)^2 + mu E:E, P = F (lambda tr(E) I + 2 mu E)
//   dP_ij/dF_kl = d_ik S_lj + lambda F_ij F_kl + mu (F_il F_kj + (F F^T)_ik d_jl)
void stvk(double lam, double mu, const double* F, double* psi, double* P, double* D) {
  double C[9], B[9];
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 3; ++i) {
      double c = 0, b = 0;
      for (int k = 0; k < 3; ++k) {
        c += F[k + 3 * i] * F[k + 3 * j];  // (F^T F)_ij
        b += F[i + 3 * k] * F[j + 3 * k];  // (F F^T)_ij
      }
      C[i + 3 * j] = c;
      B[i + 3 * j] = b;
    }
  double E[9];
  for (int a = 0; a < 9; ++a) E[a] = 0.5 * C[a];
  E[0] -= 0.5; E[4] -= 0.5; E[8] -= 0.5;
  double trE = E[0] + E[4] + E[8];
  if (psi) {
    double ee = 0;
    for (int a = 0; a < 9; ++a) ee += E[a] * E[a];
    *psi = 0.5 * lam * trE * trE + mu * ee;
  }
  double S[9];
  for (int a = 0; a < 9; ++a) S[a] = 2.0 * mu * E[a];
  S[0] += lam * trE; S[4] += lam * trE; S[8] += lam * trE;
  if (P) {
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        double v = 0;
        for (int k = 0; k < 3; ++k) v += F[i + 3 * k] * S[k + 3 * j];
        P[i + 3 * j] = v;
      }
  }
  if (D) {
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i)
        for (int l = 0; l < 3; ++l)
          for (int k = 0; k < 3; ++k) {
            double v = lam * F[i + 3 * j] * F[k + 3 * l] + mu * F[i + 3 * l] * F[k + 3 * j];
            if (i == k) v += S[l + 3 * j];
            if (j == l) v += mu * B[i + 3 * k];
            D[(i + 3 * j) * 9 + (k + 3 * l)] = v;
          }
  }
}

void material(int model, double lam, double mu, const double* F, double* psi, double* P, double* D) {
  if (model == 1)
    stvk(lam, mu, F, psi, P, D);
  else
    conh(lam, mu, F, psi, P, D);
}

// ---------------------------------------------------------------------------
// Per-element rest data: ShapeFunction_LERP::InitDeformationAtSamples with the
// Tet4 partials B = [-1 -1 -1; I] and one quadrature point of weight 1/6.
// ---------------------------------------------------------------------------
struct ElemRest {
  double DFDx[9][12];  // vec(F) = DFDx vec(Nx), column d = 3*node + comp
  double w;            // quadrature weight * det J = rest volume
  double vol0;         // VolumeBasis(Position_0), used by the lumped mass
};

bool inv3(const double* A, double* Ainv) {
  double d = det3(A);
  if (d == 0.0) return false;
  double C[9];
  cofactor3(A, C);
  // inverse = adj / det = cof^T / det
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ainv[i + 3 * j] = C[j + 3 * i] / d;
  return true;
}

}  // namespace

// ---------------------------------------------------------------------------
// Sparse LDL^T (up-looking, simplicial) with a geometric nested-dissection order
// ---------------------------------------------------------------------------
namespace {

struct LDL {
  int n = 0;
  std::vector<int> perm, pinv;         // perm[new] = old
  std::vector<int> Cp, Ci;             // permuted upper-triangular pattern (col k: rows <= k)
  std::vector<int> Cmap;               // Cmap[q] = index into the lower CSC value array
  std::vector<int> parent, Lnz, Lp;    // elimination tree, column counts, column pointers
  std::vector<int> Li;
  std::vector<double> Lx, D;
  bool analysed = false;
};

// Recursive coordinate bisection with vertex separators on the node graph.
void nd_order(const std::vector<double>& X0, const std::vector<std::vector<int>>& adj,
              std::vector<int>& nodes, std::vector<int>& out, std::vector<int>& side) {
  if (nodes.size() <= 48) {
    std::sort(nodes.begin(), nodes.end());
    out.insert(out.end(), nodes.begin(), nodes.end());
    return;
  }
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int v : nodes)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], X0[3 * v + d]);
      hi[d] = std::max(hi[d], X0[3 * v + d]);
    }
  int ax = 0;
  for (int d = 1; d < 3; ++d)
    if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
  std::sort(nodes.begin(), nodes.end(), [&](int a, int b) {
    double xa = X0[3 * a + ax], xb = X0[3 * b + ax];
    return xa < xb || (xa == xb && a < b);
  });
  size_t half = nodes.size() / 2;
  // side: 1 = left half, 2 = right half, 3 = separator, 0 = outside this subproblem
  for (size_t i = 0; i < nodes.size(); ++i) side[nodes[i]] = i < half ? 1 : 2;
  std::vector<int> A, B, S;
  for (size_t i = 0; i < half; ++i) {
    int v = nodes[i];
    bool sep = false;
    for (int u : adj[v])
      if (side[u] == 2) { sep = true; break; }
    if (sep) S.push_back(v); else A.push_back(v);
  }
  for (size_t i = half; i < nodes.size(); ++i) B.push_back(nodes[i]);
  for (int v : nodes) side[v] = 0;
  if (A.empty() || B.empty()) {  // degenerate split: emit as is
    std::sort(nodes.begin(), nodes.end());
    out.insert(out.end(), nodes.begin(), nodes.end());
    return;
  }
  nd_order(X0, adj, A, out, side);
  nd_order(X0, adj, B, out, side);
  std::sort(S.begin(), S.end());
  out.insert(out.end(), S.begin(), S.end());
}

}  // namespace

// ---------------------------------------------------------------------------
// The oracle handle
// ---------------------------------------------------------------------------
struct orc_handle_s {
  int n = 0, m = 0, N = 0;
  std::vector<double> X0;
  std::vector<int> T;
  std::vector<double> lame, rho;
  std::vector<uint8_t> model, fixed;
  std::vector<double> soft_k, soft_t;  // BC_FixDoF soft mode: [n] stiffness, [3n] targets
  std::vector<double> force;
  double grav[3] = {0, 0, 0};
  std::vector<ElemRest> rest;
  std::vector<double> nodemass;  // lumped mass per node (sum over elements, element order)

  // Lower CSC pattern of the Hessian (Eigen SparseMatrix<double> column-major)
  std::vector<int> colptr, rowidx;
  // for each tet, 10 blocks x 9 entries -> CSC value index (the reference's pointer map)
  std::vector<int> emap;  // [m][10][9]

  LDL ldl;
  std::vector<double> log_obj, log_opt, log_step;
  std::vector<int> log_bis;

  // element buffers
  std::vector<double> Ee, ge, He;

  // staged loading (BCondition stages): groups, their start values, the stage counter
  struct Group {
    int num_stages, soft;
    double k0, k1, M[9], b[3];
    std::vector<int> nodes;
    std::vector<double> ini;  // [3 * nodes]
  };
  std::vector<Group> groups;
  int num_stages = 0, stage = 0;

  // cg_parallel: full rows of the lower pattern (built once), for the row-parallel CG
  int cg_par = 0;
  std::vector<int64_t> fr_ptr;
  std::vector<int> fr_col;
  std::vector<int64_t> fr_src;  // index of each row entry in the lower CSC values
};

namespace {

// local node pairs in the reference's propagate order: i = 0..3, j = 0..i
const int kPairI[10] = {0, 1, 1, 2, 2, 2, 3, 3, 3, 3};
const int kPairJ[10] = {0, 0, 1, 0, 1, 2, 0, 1, 2, 3};

void element_rest(orc_handle_s* h) {
  h->rest.resize(h->m);
  h->nodemass.assign(h->n, 0.0);
  for (int e = 0; e < h->m; ++e) {
    const int* t = &h->T[4 * e];
    double Jm[9];  // N0 * B = [x1-x0, x2-x0, x3-x0]
    for (int c = 0; c < 3; ++c)
      for (int r = 0; r < 3; ++r) Jm[r + 3 * c] = h->X0[3 * t[c + 1] + r] - h->X0[3 * t[0] + r];
    double Ji[9];
    inv3(Jm, Ji);
    // BH0 = B * J^-1 (4x3)
    const double B[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double BH0[4][3];
    for (int a = 0; a < 4; ++a)
      for (int c = 0; c < 3; ++c) {
        double v = 0;
        for (int k = 0; k < 3; ++k) v += B[a][k] * Ji[k + 3 * c];
        BH0[a][c] = v;
      }
    ElemRest& R = h->rest[e];
    // DFDx column d: vec(E_d * BH0), E_d the 3x4 unit matrix with data()[d] = 1
    for (int d = 0; d < 12; ++d) {
      int node = d / 3, comp = d % 3;
      for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) R.DFDx[r + 3 * c][d] = (r == comp) ? BH0[node][c] : 0.0;
    }
    R.w = (1.0 / 6.0) * det3(Jm);
    R.vol0 = (1.0 / 6.0) * det3(Jm);
  }
  // MassElement_Lumped::ComputeAndStore_Mass: rho * V / 4 per node of each tet
  for (int e = 0; e < h->m; ++e) {
    double me = h->rho[e] * h->rest[e].vol0 / 4.0;
    for (int a = 0; a < 4; ++a) h->nodemass[h->T[4 * e + a]] += me;
  }
}

inline void element_F(const orc_handle_s* h, int e, const double* x, double* Fv) {
  const ElemRest& R = h->rest[e];
  double vNx[12];
  for (int a = 0; a < 4; ++a)
    for (int c = 0; c < 3; ++c) vNx[3 * a + c] = x[3 * h->T[4 * e + a] + c];
  for (int r = 0; r < 9; ++r) {
    double v = 0;
    for (int d = 0; d < 12; ++d) v += R.DFDx[r][d] * vNx[d];
    Fv[r] = v;
  }
}

inline double element_volume(const orc_handle_s* h, int e, const double* x) {
  const int* t = &h->T[4 * e];
  double M[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) M[r + 3 * c] = x[3 * t[c + 1] + r] - x[3 * t[0] + r];
  return (1.0 / 6.0) * det3(M);
}

// EnergyElement_FEM::ComputeAndStore_{Energy,Gradient,Hessian}_Internal
void element_eval(const orc_handle_s* h, int e, const double* x, double* E, double* g, double* H) {
  double Fv[9];
  element_F(h, e, x, Fv);
  const ElemRest& R = h->rest[e];
  double lam = h->lame[2 * e], mu = h->lame[2 * e + 1];
  int mdl = h->model[e];
  if (E) {
    if (element_volume(h, e, x) < 0) {
      *E = HUGE_VAL;  // inverted element (EnergyElement_FEM.cpp:126-131)
    } else {
      double psi;
      material(mdl, lam, mu, Fv, &psi, nullptr, nullptr);
      *E = 0.0 + psi * R.w;
    }
  }
  if (g) {
    double P[9];
    material(mdl, lam, mu, Fv, nullptr, P, nullptr);
    for (int d = 0; d < 12; ++d) {
      double v = 0;
      for (int r = 0; r < 9; ++r) v += R.DFDx[r][d] * P[r];
      g[d] = v * R.w;
    }
  }
  if (H) {
    double D[81];
    material(mdl, lam, mu, Fv, nullptr, nullptr, D);
    double TD[12][9];  // DFDx^T * dPdF
    for (int d = 0; d < 12; ++d)
      for (int b = 0; b < 9; ++b) {
        double v = 0;
        for (int a = 0; a < 9; ++a) v += R.DFDx[a][d] * D[a * 9 + b];
        TD[d][b] = v;
      }
    for (int d = 0; d < 12; ++d)
      for (int q = 0; q < 12; ++q) {
        double v = 0;
        for (int b = 0; b < 9; ++b) v += TD[d][b] * R.DFDx[b][q];
        H[d * 12 + q] = v * R.w;
      }
  }
}

// Builds the lower CSC pattern the way AMatrixSd's first (triplet) assembly does:
// for each tet and local pair (i, j<=i), block rows go to max(off_i, off_j); diagonal
// node blocks are stored in full; duplicates are summed, structural zeros kept.
void build_pattern(orc_handle_s* h) {
  int N = h->N;
  std::vector<std::vector<int>> cols(N);
  for (int e = 0; e < h->m; ++e)
    for (int p = 0; p < 10; ++p) {
      int ni = h->T[4 * e + kPairI[p]], nj = h->T[4 * e + kPairJ[p]];
      int R = std::max(ni, nj), C = std::min(ni, nj);
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) cols[3 * C + b].push_back(3 * R + a);
    }
  h->colptr.assign(N + 1, 0);
  for (int c = 0; c < N; ++c) {
    auto& v = cols[c];
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    h->colptr[c + 1] = h->colptr[c] + (int)v.size();
  }
  h->rowidx.resize(h->colptr[N]);
  for (int c = 0; c < N; ++c) std::copy(cols[c].begin(), cols[c].end(), h->rowidx.begin() + h->colptr[c]);
  // pointer map (AMatrixSd::CreateBlock): element block entry -> CSC index
  h->emap.resize((size_t)h->m * 90);
  for (int e = 0; e < h->m; ++e)
    for (int p = 0; p < 10; ++p) {
      int li = kPairI[p], lj = kPairJ[p];
      int oi = 3 * h->T[4 * e + li], oj = 3 * h->T[4 * e + lj];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
          // local block entry (a, b) of H(3li.., 3lj..) goes to (oi+a, oj+b) or its transpose
          int r = oi + a, c = oj + b;
          if (oi < oj) std::swap(r, c);
          const int* beg = &h->rowidx[h->colptr[c]];
          const int* end = &h->rowidx[h->colptr[c + 1]];
          const int* it = std::lower_bound(beg, end, r);
          h->emap[(size_t)e * 90 + p * 9 + a * 3 + b] = (int)(it - h->rowidx.data());
        }
    }
}

void ensure_elem_buffers(orc_handle_s* h) {
  if ((int)h->Ee.size() != h->m) {
    h->Ee.resize(h->m);
    h->ge.resize((size_t)h->m * 12);
    h->He.resize((size_t)h->m * 144);
  }
}

struct Timers {
  double cal_ene = 0, cal_gra = 0, cal_hes = 0, ass_gra = 0, ass_hes = 0, opt_sol = 0, opt_lis = 0;
};

// Simulable::AddEnergy: elements in order, then lumped-mass gravity, then force BCs.
double model_energy(orc_handle_s* h, const double* x, Timers* tm) {
  ensure_elem_buffers(h);
  auto t0 = clk::now();
#pragma omp parallel for schedule(static)
  for (int e = 0; e < h->m; ++e) element_eval(h, e, x, &h->Ee[e], nullptr, nullptr);
  auto t1 = clk::now();
  double E = 0;
  for (int e = 0; e < h->m; ++e) E += h->Ee[e];
  bool grav = h->grav[0] != 0 || h->grav[1] != 0 || h->grav[2] != 0;
  if (grav) {
    for (int e = 0; e < h->m; ++e) {
      double me = h->rho[e] * h->rest[e].vol0 / 4.0;
      double v = 0;
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 3; ++c) v += x[3 * h->T[4 * e + a] + c] * (-me * h->grav[c]);
      E += v;
    }
  } else {
    E += 0.0;
  }
  if (!h->force.empty())
    for (int i = 0; i < h->n; ++i) {
      double v = 0;
      for (int c = 0; c < 3; ++c) v += x[3 * i + c] * h->force[3 * i + c];
      E += v;
    }
  // BC_FixDoF soft mode: EnergyElement_SoftConstraint::ComputeAndStore_Energy_Internal
  // (EnergyElement_SoftConstraint.cpp:45-53), 0.5 k c.c with c = x - t
  // (ConstraintSet_FixedPosition.cpp:44-46)
  if (!h->soft_k.empty())
    for (int i = 0; i < h->n; ++i) {
      if (h->soft_k[i] == 0.0) continue;
      double cc = 0;
      for (int c = 0; c < 3; ++c) {
        double d = x[3 * i + c] - h->soft_t[3 * i + c];
        cc += d * d;
      }
      E += 0.5 * h->soft_k[i] * cc;
    }
  if (tm) tm->cal_ene += secs(t0, t1);
  return E;
}

// Simulable::GetGradient (+ FixVectorDoFs when fix != 0)
void model_gradient(orc_handle_s* h, const double* x, double* g, bool fix, Timers* tm) {
  ensure_elem_buffers(h);
  auto t0 = clk::now();
#pragma omp parallel for schedule(static)
  for (int e = 0; e < h->m; ++e) element_eval(h, e, x, nullptr, &h->ge[(size_t)e * 12], nullptr);
  auto t1 = clk::now();
  std::fill(g, g + h->N, 0.0);
  for (int e = 0; e < h->m; ++e)
    for (int a = 0; a < 4; ++a)
      for (int c = 0; c < 3; ++c) g[3 * h->T[4 * e + a] + c] += h->ge[(size_t)e * 12 + 3 * a + c];
  bool grav = h->grav[0] != 0 || h->grav[1] != 0 || h->grav[2] != 0;
  if (grav)
    for (int e = 0; e < h->m; ++e) {
      double me = h->rho[e] * h->rest[e].vol0 / 4.0;
      for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 3; ++c) g[3 * h->T[4 * e + a] + c] += -me * h->grav[c];
    }
  if (!h->force.empty())
    for (int i = 0; i < h->N; ++i) g[i] += h->force[i];
  if (!h->soft_k.empty())  // k J^T c with J = I (EnergyElement_SoftConstraint.cpp:55-66)
    for (int i = 0; i < h->n; ++i)
      for (int c = 0; c < 3; ++c) g[3 * i + c] += h->soft_k[i] * (x[3 * i + c] - h->soft_t[3 * i + c]);
  if (fix && !h->fixed.empty())
    for (int i = 0; i < h->N; ++i)
      if (h->fixed[i]) g[i] = 0.0;
  auto t2 = clk::now();
  if (tm) { tm->cal_gra += secs(t0, t1); tm->ass_gra += secs(t1, t2); }
}

// Simulable::GetHessian through the pointer map (+ FixMatrixDoFs when fix != 0)
void model_hessian(orc_handle_s* h, const double* x, double* vals, bool fix, Timers* tm) {
  ensure_elem_buffers(h);
  auto t0 = clk::now();
#pragma omp parallel for schedule(static)
  for (int e = 0; e < h->m; ++e) element_eval(h, e, x, nullptr, nullptr, &h->He[(size_t)e * 144]);
  auto t1 = clk::now();
  size_t nnz = h->rowidx.size();
  std::fill(vals, vals + nnz, 0.0);
  for (int e = 0; e < h->m; ++e) {
    const double* He = &h->He[(size_t)e * 144];
    const int* mp = &h->emap[(size_t)e * 90];
    for (int p = 0; p < 10; ++p) {
      int li = kPairI[p], lj = kPairJ[p];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) vals[mp[p * 9 + a * 3 + b]] += He[(3 * li + a) * 12 + 3 * lj + b];
    }
  }
  if (!h->soft_k.empty())  // k J^T J = k I on the node's diagonal (EnergyElement_SoftConstraint.cpp:68-86)
    for (int c = 0; c < h->N; ++c) {
      const double k = h->soft_k[c / 3];
      if (k == 0.0) continue;
      for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q)
        if (h->rowidx[q] == c) vals[q] += k;
    }
  if (fix && !h->fixed.empty())
    for (int c = 0; c < h->N; ++c)
      for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q) {
        int r = h->rowidx[q];
        if (h->fixed[r] || h->fixed[c]) vals[q] = (r == c) ? 1.0 : 0.0;
      }
  auto t2 = clk::now();
  if (tm) { tm->cal_hes += secs(t0, t1); tm->ass_hes += secs(t1, t2); }
}

double norm2(const double* v, int n) {
  double s = 0;
  for (int i = 0; i < n; ++i) s += v[i] * v[i];
  return std::sqrt(s);
}

// y = A x with A = selfadjointView<Lower>() of the stored lower CSC
void symv_lower(const orc_handle_s* h, const double* vals, const double* x, double* y) {
  int N = h->N;
  std::fill(y, y + N, 0.0);
  for (int c = 0; c < N; ++c)
    for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q) {
      int r = h->rowidx[q];
      if (r < c) continue;
      y[r] += vals[q] * x[c];
      if (r != c) y[c] += vals[q] * x[r];
    }
}

// LinearSolver::GetMatrixData (LinearSolver.cpp:57-66): Frobenius norm of the stored entries
void matrix_data(const std::vector<double>& vals, double* normA, double* sinT, double* regT) {
  double s = 0;
  for (double v : vals) s += v * v;
  *normA = std::sqrt(s);
  *sinT = std::max(std::min(1e-6 * *normA, 1e-6), 1e-9);
  *regT = 1e-6 * *normA;
}

void add_identity(const orc_handle_s* h, std::vector<double>& vals, double s) {
  for (int c = 0; c < h->N; ++c)
    for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q)
      if (h->rowidx[q] == c) vals[q] += s;
}

// ---- LDL^T --------------------------------------------------------------
void ldl_analyse(orc_handle_s* h) {
  LDL& L = h->ldl;
  int N = h->N;
  L.n = N;
  // node graph for the ordering
  std::vector<std::vector<int>> adj(h->n);
  for (int e = 0; e < h->m; ++e)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 4; ++b)
        if (a != b) adj[h->T[4 * e + a]].push_back(h->T[4 * e + b]);
  for (auto& v : adj) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
  }
  std::vector<int> nodes(h->n), order, side(h->n, 0);
  std::iota(nodes.begin(), nodes.end(), 0);
  nd_order(h->X0, adj, nodes, order, side);
  L.perm.resize(N);
  for (int i = 0; i < h->n; ++i)
    for (int c = 0; c < 3; ++c) L.perm[3 * i + c] = 3 * order[i] + c;
  L.pinv.resize(N);
  for (int k = 0; k < N; ++k) L.pinv[L.perm[k]] = k;
  // permuted upper pattern from the stored lower entries (row >= col only)
  std::vector<int> cnt(N + 1, 0);
  for (int c = 0; c < N; ++c)
    for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q) {
      int r = h->rowidx[q];
      if (r < c) continue;
      int pr = L.pinv[r], pc = L.pinv[c];
      cnt[std::max(pr, pc) + 1]++;
    }
  for (int k = 0; k < N; ++k) cnt[k + 1] += cnt[k];
  L.Cp = cnt;
  L.Ci.resize(cnt[N]);
  L.Cmap.resize(cnt[N]);
  std::vector<int> pos(cnt.begin(), cnt.end() - 1);
  for (int c = 0; c < N; ++c)
    for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q) {
      int r = h->rowidx[q];
      if (r < c) continue;
      int pr = L.pinv[r], pc = L.pinv[c];
      int col = std::max(pr, pc), row = std::min(pr, pc);
      int at = pos[col]++;
      L.Ci[at] = row;
      L.Cmap[at] = q;
    }
  // elimination tree and column counts (LDL symbolic)
  L.parent.assign(N, -1);
  L.Lnz.assign(N, 0);
  std::vector<int> flag(N, -1);
  for (int k = 0; k < N; ++k) {
    flag[k] = k;
    for (int p = L.Cp[k]; p < L.Cp[k + 1]; ++p) {
      int i = L.Ci[p];
      if (i < k) {
        for (; flag[i] != k; i = L.parent[i]) {
          if (L.parent[i] == -1) L.parent[i] = k;
          L.Lnz[i]++;
          flag[i] = k;
        }
      }
    }
  }
  L.Lp.assign(N + 1, 0);
  for (int k = 0; k < N; ++k) L.Lp[k + 1] = L.Lp[k] + L.Lnz[k];
  L.Li.resize(L.Lp[N]);
  L.Lx.resize(L.Lp[N]);
  L.D.resize(N);
  L.analysed = true;
}

// numeric factorisation; returns the first k with D[k] == 0, or -1
int ldl_factor(orc_handle_s* h, const std::vector<double>& vals) {
  LDL& L = h->ldl;
  int N = L.n;
  std::vector<double> Y(N, 0.0);
  std::vector<int> pattern(N), flag(N), lnz(N, 0);
  for (int k = 0; k < N; ++k) {
    Y[k] = 0.0;
    int top = N;
    flag[k] = k;
    lnz[k] = 0;
    for (int p = L.Cp[k]; p < L.Cp[k + 1]; ++p) {
      int i = L.Ci[p];
      Y[i] += vals[L.Cmap[p]];
      int len = 0;
      for (; flag[i] != k; i = L.parent[i]) {
        pattern[len++] = i;
        flag[i] = k;
      }
      while (len > 0) pattern[--top] = pattern[--len];
    }
    L.D[k] = Y[k];
    Y[k] = 0.0;
    for (; top < N; ++top) {
      int i = pattern[top];
      double yi = Y[i];
      Y[i] = 0.0;
      int p2 = L.Lp[i] + lnz[i];
      for (int p = L.Lp[i]; p < p2; ++p) Y[L.Li[p]] -= L.Lx[p] * yi;
      double l_ki = yi / L.D[i];
      L.D[k] -= l_ki * yi;
      L.Li[p2] = k;
      L.Lx[p2] = l_ki;
      lnz[i]++;
    }
    if (L.D[k] == 0.0) return k;
  }
  return -1;
}

void ldl_solve(const orc_handle_s* h, const double* b, double* x) {
  const LDL& L = h->ldl;
  int N = L.n;
  std::vector<double> y(N);
  for (int k = 0; k < N; ++k) y[k] = b[L.perm[k]];
  for (int j = 0; j < N; ++j)
    for (int p = L.Lp[j]; p < L.Lp[j + 1]; ++p) y[L.Li[p]] -= L.Lx[p] * y[j];
  for (int j = 0; j < N; ++j) y[j] /= L.D[j];
  for (int j = N - 1; j >= 0; --j)
    for (int p = L.Lp[j]; p < L.Lp[j + 1]; ++p) y[j] -= L.Lx[p] * y[L.Li[p]];
  for (int k = 0; k < N; ++k) x[L.perm[k]] = y[k];
}

// LinearSolver_EigenLDLT::SolveInternal (LinearSolver_EigenLDLT.cpp:49-154)
int solve_ldlt(orc_handle_s* h, std::vector<double>& A, const std::vector<double>& b,
               std::vector<double>& x, double maxError, int regIters, int* regUsed) {
  int N = h->N;
  if (!h->ldl.analysed) ldl_analyse(h);
  double normA, sinT, regT;
  matrix_data(A, &normA, &sinT, &regT);
  std::vector<double> bt(N);
  double bn = norm2(b.data(), N);
  for (int i = 0; i < regIters; ++i) {
    if (i != 0) {
      add_identity(h, A, regT * std::pow(10.0, i - 1));
      if (regUsed) (*regUsed)++;
    }
    if (ldl_factor(h, A) >= 0) continue;  // factorisation failed
    bool sing = false;
    for (int j = 0; j < N; ++j)
      if (std::fabs(h->ldl.D[j]) < sinT) { sing = true; break; }
    if (sing) continue;
    ldl_solve(h, b.data(), x.data());
    double xn = norm2(x.data(), N);
    double dot = 0;
    if (bn > 0 && xn > 0) {
      for (int j = 0; j < N; ++j) dot += (b[j] / bn) * (x[j] / xn);
    }
    if (dot < -regT) continue;
    symv_lower(h, A.data(), x.data(), bt.data());
    double ae = 0;
    for (int j = 0; j < N; ++j) ae += (b[j] - bt[j]) * (b[j] - bt[j]);
    ae = std::sqrt(ae);
    double re = ae / bn;
    if (ae > maxError && re > maxError) continue;
    return 0;  // LSResult::SUCCESS
  }
  return 1;  // LSResult::FAILURE
}

// Full rows of the symmetric matrix stored as its lower CSC: for each row, its columns in
// ascending order and where each value sits in the lower CSC array.
void full_rows(orc_handle_s* h) {
  if (!h->fr_ptr.empty()) return;
  const int N = h->N;
  std::vector<int64_t> cnt(N + 1, 0);
  for (int c = 0; c < N; ++c)
    for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q) {
      const int r = h->rowidx[q];
      if (r < c) continue;
      cnt[r + 1]++;
      if (r != c) cnt[c + 1]++;
    }
  for (int i = 0; i < N; ++i) cnt[i + 1] += cnt[i];
  h->fr_ptr = cnt;
  h->fr_col.resize(cnt[N]);
  h->fr_src.resize(cnt[N]);
  std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
  // columns ascending per row: entries (r, c) with c < r come from columns c < r in order, then
  // the diagonal, then the transposed entries (c, r) with r > c, in increasing row order
  for (int c = 0; c < N; ++c)
    for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q) {
      const int r = h->rowidx[q];
      if (r < c) continue;
      if (r != c) { h->fr_col[pos[r]] = c; h->fr_src[pos[r]++] = q; }
    }
  for (int c = 0; c < N; ++c)
    for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q) {
      const int r = h->rowidx[q];
      if (r < c) continue;
      h->fr_col[pos[c]] = r;
      h->fr_src[pos[c]++] = q;
    }
}

// Inner product in fixed blocks of 4096 entries, block sums added in order: the same bits
// for any number of threads.
double dot_blocked(const double* a, const double* b, int N) {
  const int nb = (N + 4095) / 4096;
  std::vector<double> part(nb);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < nb; ++k) {
    double s = 0;
    const int i1 = std::min(N, (k + 1) * 4096);
    for (int i = k * 4096; i < i1; ++i) s += a[i] * b[i];
    part[k] = s;
  }
  double s = 0;
  for (double v : part) s += v;
  return s;
}

// Jacobi / block-Jacobi preconditioned CG with Eigen's ConjugateGradient rules.  With
// h->cg_par the products run row-parallel over full rows and the inner products in fixed
// blocks (the same iteration, summed in another order; used for systems of millions of DoFs).
int64_t pcg(const orc_handle_s* h, const std::vector<double>& A, const std::vector<double>& b,
            std::vector<double>& x, double tol, int maxIters, bool block) {
  int N = h->N;
  const bool par = h->cg_par != 0;
  auto mv = [&](const double* in, double* out) {
    if (!par) { symv_lower(h, A.data(), in, out); return; }
#pragma omp parallel for schedule(static, 1024)
    for (int r = 0; r < N; ++r) {
      double s = 0;
      for (int64_t k = h->fr_ptr[r]; k < h->fr_ptr[r + 1]; ++k) s += A[h->fr_src[k]] * in[h->fr_col[k]];
      out[r] = s;
    }
  };
  auto dot = [&](const std::vector<double>& a, const std::vector<double>& c) {
    if (par) return dot_blocked(a.data(), c.data(), N);
    double s = 0;
    for (int i = 0; i < N; ++i) s += a[i] * c[i];
    return s;
  };
  std::vector<double> inv(block ? (size_t)N * 3 : (size_t)N, 0.0);
  if (!block) {
    for (int c = 0; c < N; ++c) {
      inv[c] = 1.0;
      for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q)
        if (h->rowidx[q] == c && A[q] != 0.0) inv[c] = 1.0 / A[q];
    }
  } else {
    for (int v = 0; v < h->n; ++v) {
      double Bk[9];
      for (int b2 = 0; b2 < 3; ++b2) {
        int c = 3 * v + b2;
        for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q) {
          int r = h->rowidx[q];
          if (r >= 3 * v && r < 3 * v + 3 && r >= c) {
            Bk[(r - 3 * v) + 3 * b2] = A[q];
            Bk[b2 + 3 * (r - 3 * v)] = A[q];
          }
        }
      }
      double Bi[9];
      if (!inv3(Bk, Bi)) { for (int a = 0; a < 9; ++a) Bi[a] = (a % 4 == 0) ? 1.0 : 0.0; }
      for (int a = 0; a < 9; ++a) inv[(size_t)9 * v + a] = Bi[a];
    }
  }
  auto apply = [&](const std::vector<double>& r, std::vector<double>& z) {
    if (!block) {
#pragma omp parallel for schedule(static) if (par)
      for (int i = 0; i < N; ++i) z[i] = inv[i] * r[i];
    } else {
#pragma omp parallel for schedule(static) if (par)
      for (int v = 0; v < h->n; ++v)
        for (int a = 0; a < 3; ++a) {
          double s = 0;
          for (int c = 0; c < 3; ++c) s += inv[(size_t)9 * v + a + 3 * c] * r[3 * v + c];
          z[3 * v + a] = s;
        }
    }
  };
  std::vector<double> r(N), z(N), p(N), q(N);
  mv(x.data(), q.data());
  for (int i = 0; i < N; ++i) r[i] = b[i] - q[i];
  double rhs2 = dot(b, b);
  if (rhs2 == 0) { std::fill(x.begin(), x.end(), 0.0); return 0; }
  double thr = std::max(tol * tol * rhs2, DBL_MIN);
  double rr = dot(r, r);
  if (rr < thr) return 0;
  apply(r, p);
  double rz = dot(r, p);
  int64_t it = 0;
  while (it < maxIters) {
    mv(p.data(), q.data());
    double pq = dot(p, q);
    double alpha = rz / pq;
#pragma omp parallel for schedule(static) if (par)
    for (int i = 0; i < N; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * q[i]; }
    rr = dot(r, r);
    if (rr < thr) { ++it; break; }
    apply(r, z);
    double rzo = rz;
    rz = dot(r, z);
    double beta = rz / rzo;
#pragma omp parallel for schedule(static) if (par)
    for (int i = 0; i < N; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  return it;
}

// LinearSolver_EigenCG::SolveInternal (LinearSolver_EigenCG.cpp:51-125)
int solve_cg(orc_handle_s* h, std::vector<double>& A, const std::vector<double>& b, std::vector<double>& x,
             double tol, int maxIters, int regIters, bool block, int* regUsed, int64_t* iters) {
  double normA, sinT, regT;
  matrix_data(A, &normA, &sinT, &regT);
  std::vector<double> xprev = x;
  for (int i = 0; i < regIters; ++i) {
    if (i != 0) {
      add_identity(h, A, regT * std::pow(10.0, i - 1));
      if (regUsed) (*regUsed)++;
    }
    x = xprev;
    int64_t it = pcg(h, A, b, x, tol, maxIters, block);
    if (iters) *iters += it;
    double dot = 0;
    for (int j = 0; j < h->N; ++j) dot += b[j] * x[j];
    if (dot < 0.0) continue;
    return 0;
  }
  return 1;
}

// ---------------------------------------------------------------------------
// Optimisation problems (static / implicit Euler) and OptimSolver::SolveFull
// ---------------------------------------------------------------------------
struct Problem {
  orc_handle_s* h;
  bool dynamic = false;
  double dt = 0;
  std::vector<double> x0, v0;  // dynamic: state at solve start
  std::vector<double> x;       // model positions (Position_X)
  std::vector<double> v;       // model velocities
  std::vector<double> saved;   // GetState snapshot (positions + velocities)
  Timers tm;

  int N() const { return h->N; }
  // dynamic: a = (x - x0)/dt^2 - v0/dt
  void accel(std::vector<double>& a) const {
    a.resize(N());
    double dt2 = dt * dt;
    for (int i = 0; i < N(); ++i) a[i] = (x[i] - x0[i]) / dt2 - v0[i] / dt;
  }
  double mass_dof(int i) const { return h->nodemass[i / 3]; }
  double energy() {
    double e = model_energy(h, x.data(), &tm);
    if (dynamic) {
      std::vector<double> a;
      accel(a);
      double s = 0;
      for (int i = 0; i < N(); ++i) s += a[i] * (mass_dof(i) * a[i]);
      e += (dt * dt / 2.0) * s;
    }
    return e;
  }
  void gradient(std::vector<double>& g) {
    g.resize(N());
    model_gradient(h, x.data(), g.data(), !dynamic, &tm);
    if (dynamic) {
      std::vector<double> a;
      accel(a);
      for (int i = 0; i < N(); ++i) g[i] += mass_dof(i) * a[i];
      if (!h->fixed.empty())
        for (int i = 0; i < N(); ++i)
          if (h->fixed[i]) g[i] = 0.0;
    }
  }
  void hessian(std::vector<double>& H) {
    H.resize(h->rowidx.size());
    model_hessian(h, x.data(), H.data(), !dynamic, &tm);
    if (dynamic) {
      add_identity_mass(H);
      if (!h->fixed.empty())
        for (int c = 0; c < N(); ++c)
          for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q) {
            int r = h->rowidx[q];
            if (h->fixed[r] || h->fixed[c]) H[q] = (r == c) ? 1.0 : 0.0;
          }
    }
  }
  void add_identity_mass(std::vector<double>& H) {
    double s = 1.0 / (dt * dt);
    for (int c = 0; c < N(); ++c)
      for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q)
        if (h->rowidx[q] == c) H[q] += mass_dof(c) * s;
  }
  void save() { saved = x; saved.insert(saved.end(), v.begin(), v.end()); }
  void restore() {
    std::copy(saved.begin(), saved.begin() + N(), x.begin());
    std::copy(saved.begin() + N(), saved.end(), v.begin());
  }
  void pos_perform_step() {
    if (dynamic)
      for (int i = 0; i < N(); ++i) v[i] = (x[i] - x0[i]) / dt;
  }
};

enum { ONGOING = 0, SUCCESS = 1, MINSTEP = 2, MINIMPR = 3, FAILURE = 4, MAXITER = 5, NONDESC = 6 };

// Simulable::StepBoundaryConditions (Simulable.cpp:1496-1500): one more stage (while not all
// boundary conditions are loaded), then each group's BC_FixDoF::Update (BC_FixDoF.cpp:80-121)
// at its own a = min(stage, N) / N: hard groups set their DoFs (positions) to the targets,
// soft groups set targets and the ramped stiffness.  VectorAnimator_LerpT3D::Evaluate
// (VectorAnimators.h:135-145) maps a start value v to (I + a Mt) [v; 1] with Mt the
// animator's 4x4 (its translation b and linear part M), i.e. a b + (I + a M) v.
bool step_stage(orc_handle_s* h, std::vector<double>& x) {
  if (h->num_stages <= 0 || h->stage >= h->num_stages) return false;
  h->stage++;
  for (auto& G : h->groups) {
    const double a = (double)std::min(h->stage, G.num_stages) / (double)G.num_stages;
    for (size_t k = 0; k < G.nodes.size(); ++k) {
      const int i = G.nodes[k];
      const double* v = &G.ini[3 * k];
      double t[3];
      for (int r = 0; r < 3; ++r)
        t[r] = a * G.b[r] + v[r] + a * (G.M[3 * r] * v[0] + G.M[3 * r + 1] * v[1] + G.M[3 * r + 2] * v[2]);
      if (G.soft) {
        for (int r = 0; r < 3; ++r) h->soft_t[3 * i + r] = t[r];
        h->soft_k[i] = G.k0 + a * (G.k1 - G.k0);
      } else {
        for (int r = 0; r < 3; ++r) x[3 * i + r] = t[r];
      }
    }
  }
  return true;
}

// OptimProblem_BasicStatic::IsFullyConstrained (OptimProblem_BasicStatic.cpp:119-121):
// Simulable::BoundaryConditionsLoaded, every condition at its last stage.
bool fully_constrained(const orc_handle_s* h) { return h->num_stages <= 1 || h->stage >= h->num_stages; }

struct State {
  std::vector<double> vx, v0, vg;
  double obj = 0, opt = 0;
  int result = SUCCESS;
  bool steepest = false;
  int minImprCount = 0, minStepCount = 0;
};

int solve_full(orc_handle_s* h, Problem& P, const orc_options* o, orc_report* rep) {
  auto tstart = clk::now();
  int N = h->N;
  State S;
  // OptimSolver::Init: variables, energy, gradient, Hessian at the initial state
  S.vx = P.x;
  S.v0 = S.vx;
  if (P.dynamic) {
    // OnSolveStart (OptimProblem_BasicDynamic.cpp:121-135): x0, v0, the boundary conditions'
    // next stage, then the predictor x = x0 + dt v0 over every DoF (hard-fixed ones included)
    P.x0 = P.x;
    P.v0 = P.v;
    step_stage(h, P.x);
    for (int i = 0; i < N; ++i) P.x[i] = P.x0[i] + P.dt * P.v0[i];
    S.vx = P.x;
    S.v0 = S.vx;
  }
  h->log_obj.clear(); h->log_opt.clear(); h->log_step.clear(); h->log_bis.clear();
  P.gradient(S.vg);
  S.opt = norm2(S.vg.data(), N);
  S.result = SUCCESS;
  S.steepest = false;
  int itCount = 0, totalBis = 0, regUsed = 0;
  int64_t linIters = 0;
  double opt0 = -1;
  std::vector<double> dx(N), dxFin(N), gNew(N), H;
  while (true) {
    itCount++;
    // ---- SolveStep -> OptimSolver_USQP_LS::SolveStepInternal
    int qp = S.steepest ? 0 : o->qp_solver;
    if (!P.dynamic) step_stage(h, P.x);  // OnIterStart: StepBoundaryConditions (static problem)
    P.save();  // OnIterStart: GetState
    S.obj = P.energy();
    P.gradient(S.vg);
    S.vx = P.x;
    S.opt = norm2(S.vg.data(), N);
    if (opt0 < 0) opt0 = S.opt;
    int numBis = 0;
    double stepNorm = 0;
    if (S.opt < o->tol_max_error) {
      S.result = SUCCESS;
    } else {
      // ComputeStep (trial 0; ComputeStep always returns true)
      auto ts = clk::now();
      if (qp == 0) {
        for (int i = 0; i < N; ++i) dx[i] = -S.vg[i];
      } else {
        P.hessian(H);
        for (int i = 0; i < N; ++i) dx[i] = S.vx[i] - S.v0[i];
        std::vector<double> b(N);
        for (int i = 0; i < N; ++i) b[i] = -S.vg[i];
        std::vector<double> xs(dx.begin(), dx.end());
        if (o->ls_solver == 1)
          solve_cg(h, H, b, xs, o->ls_tol_max_error, o->ls_num_max_iters, 10, o->cg_block_jacobi != 0,
                   &regUsed, &linIters);
        else
          solve_ldlt(h, H, b, xs, o->ls_tol_max_error, 10, &regUsed);
        std::copy(xs.begin(), xs.end(), dx.begin());
      }
      double len = norm2(dx.data(), N);
      if (len > o->max_step_size)
        for (int i = 0; i < N; ++i) dx[i] = (dx[i] / len) * o->max_step_size;
      auto te = clk::now();
      P.tm.opt_sol += secs(ts, te);
      // LineSearch_{None,Simple,Armijo,WolfeWeak,WolfeStrong} (OptimSolver.cpp:688-900).
      // m = dxIn . g with dxIn the clamped step; Armijo uses dxIn normalised (Eigen's
      // normalized() leaves a zero vector as it is).
      const int lst = o->lsearch_type;
      double m = 0;
      for (int i = 0; i < N; ++i) m += dx[i] * S.vg[i];
      const double dlen = norm2(dx.data(), N);
      const double tArm = o->lsearch_wolfe1 * (dlen > 0 ? m / dlen : 0.0);
      const double t1 = o->lsearch_wolfe1 * m, t2 = -o->lsearch_wolfe2 * m, t3 = o->lsearch_wolfe2 * std::fabs(m);
      double factor = 1.0, objNew = 0;
      bool improved = false;
      P.restore();
      if (lst == 0) {  // LineSearch_None: the full step, whatever it does
        for (int i = 0; i < N; ++i) dxFin[i] = dx[i];
        for (int i = 0; i < N; ++i) P.x[i] += dxFin[i];
        P.pos_perform_step();
        objNew = P.energy();
        P.gradient(gNew);
        numBis = 0;
        improved = true;
      } else {
        numBis = -1;
        do {
          numBis++;
          for (int i = 0; i < N; ++i) dxFin[i] = factor * dx[i];
          for (int i = 0; i < N; ++i) P.x[i] += dxFin[i];
          P.pos_perform_step();
          objNew = P.energy();
          P.gradient(gNew);
          double dgn = 0;
          for (int i = 0; i < N; ++i) dgn += dx[i] * gNew[i];
          bool ok;
          if (lst == 2) ok = objNew <= S.obj + factor * tArm;
          else if (lst == 3) ok = objNew <= S.obj + factor * t1 && -dgn <= t2;
          else if (lst == 4) ok = objNew <= S.obj + factor * t1 && -dgn <= t2 && std::fabs(dgn) <= t3;
          else ok = objNew < S.obj;
          if (ok) { improved = true; break; }
          factor *= o->lsearch_alpha;
          P.restore();
        } while (norm2(dxFin.data(), N) > o->tol_min_step && numBis <= o->lsearch_num_try);
      }
      (void)improved;  // UpdateStepResult judges the last trial by its energy alone
      P.tm.opt_lis += secs(te, clk::now());
      // UpdateStepResult
      double impr = S.obj - objNew;
      double step = norm2(dxFin.data(), N);
      stepNorm = step;
      if (impr > 0) {
        double optNew = norm2(gNew.data(), N);
        if (impr < o->tol_min_impr) {
          S.minImprCount++;
          S.result = MINIMPR;
        } else if (step < o->tol_min_step) {
          S.minStepCount++;
          S.result = MINSTEP;
        } else if (optNew <= o->tol_max_error) {
          S.result = SUCCESS;
          S.minImprCount = 0;
          S.minStepCount = 0;
        } else {
          S.result = ONGOING;
          S.minImprCount = 0;
          S.minStepCount = 0;
        }
        S.v0 = S.vx;
        for (int i = 0; i < N; ++i) S.vx[i] += dxFin[i];
        S.vg = gNew;
        S.obj = objNew;
        S.opt = optNew;
      } else {
        S.result = NONDESC;
      }
    }
    totalBis += std::max(numBis, 0);
    h->log_obj.push_back(S.obj);
    h->log_opt.push_back(S.opt);
    h->log_bis.push_back(numBis);
    h->log_step.push_back(stepNorm);
    // ---- back in SolveFull
    P.gradient(S.vg);
    S.opt = norm2(S.vg.data(), N);
    // SolveFull applies its stop rules only while IsFullyConstrained (OptimSolver.cpp:213):
    // always for the dynamic problem, once every stage is loaded for the static one
    bool brk = false;
    const bool loaded = P.dynamic || fully_constrained(h);
    if (!loaded) {
      // no rule applies; the result of the step stays as it is
    } else if (S.result == NONDESC) {
      if (!o->try_steepest) brk = true;
      else if (S.steepest) brk = true;
      else S.steepest = true;
    }
    if (loaded && !brk && S.result == MINIMPR) {
      if (S.minImprCount == o->min_impr_max_count) brk = true;
      else if (o->try_steepest) S.steepest = !S.steepest;
    }
    if (loaded && !brk && S.result == MINSTEP) {
      if (S.minStepCount == o->min_step_max_count) brk = true;
      else if (o->try_steepest) S.steepest = !S.steepest;
    }
    if (loaded && !brk && S.result == SUCCESS) {
      if (S.opt <= o->tol_max_error) brk = true;
      else S.result = ONGOING;
    }
    if (loaded && !brk && S.result == ONGOING) S.steepest = false;
    if (brk) break;
    if (itCount + 1 > o->num_max_iters) {
      S.result = MAXITER;
      break;
    }
  }
  if (rep) {
    rep->result = S.result;
    rep->iterations = itCount;
    rep->bisections = totalBis;
    rep->reg_trials = regUsed;
    rep->lin_iterations = linIters;
    rep->obj = S.obj;
    rep->opt = S.opt;
    rep->opt0 = opt0;
    rep->seconds = secs(tstart, clk::now());
    rep->t_cal_ene = P.tm.cal_ene; rep->t_cal_gra = P.tm.cal_gra; rep->t_cal_hes = P.tm.cal_hes;
    rep->t_ass_gra = P.tm.ass_gra; rep->t_ass_hes = P.tm.ass_hes;
    rep->t_opt_sol = P.tm.opt_sol; rep->t_opt_lis = P.tm.opt_lis;
  }
  return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// C API
// ---------------------------------------------------------------------------
extern "C" {

void orc_default_options(orc_options* o) {
  o->qp_solver = 1;
  o->tol_max_error = 1e-6;
  o->tol_min_step = 1e-5;
  o->min_step_max_count = 3;
  o->tol_min_impr = 1e-9;
  o->min_impr_max_count = 3;
  o->num_max_iters = 100;
  o->try_steepest = 1;
  o->max_step_size = 1000;
  o->ls_solver = 2;
  o->ls_num_max_iters = 1000;
  o->ls_tol_max_error = 1e-9;
  o->ls_num_reg_trials = 10;
  o->lsearch_type = 1;
  o->lsearch_alpha = 0.5;
  o->lsearch_num_try = 32;
  o->lsearch_wolfe1 = 1e-4;
  o->lsearch_wolfe2 = 0.9;
  o->cg_block_jacobi = 0;
  o->threads = 0;
  o->cg_parallel = 0;
}

int orc_create(const orc_mesh* mesh, orc_handle* out) {
  if (!mesh || !out || mesh->n <= 0 || mesh->m <= 0 || !mesh->X0 || !mesh->T || !mesh->lame ||
      !mesh->rho || !mesh->model)
    return -1;
  for (int64_t i = 0; i < 4LL * mesh->m; ++i)
    if (mesh->T[i] < 0 || mesh->T[i] >= mesh->n) return -1;
  auto* h = new orc_handle_s();
  h->n = mesh->n;
  h->m = mesh->m;
  h->N = 3 * mesh->n;
  h->X0.assign(mesh->X0, mesh->X0 + h->N);
  h->T.assign(mesh->T, mesh->T + 4 * (size_t)h->m);
  h->lame.assign(mesh->lame, mesh->lame + 2 * (size_t)h->m);
  h->rho.assign(mesh->rho, mesh->rho + h->m);
  h->model.assign(mesh->model, mesh->model + h->m);
  if (mesh->fixed) h->fixed.assign(mesh->fixed, mesh->fixed + h->N);
  if (mesh->force) h->force.assign(mesh->force, mesh->force + h->N);
  for (int c = 0; c < 3; ++c) h->grav[c] = mesh->gravity[c];
  if (mesh->soft_k) {
    h->soft_k.assign(mesh->soft_k, mesh->soft_k + h->n);
    const double* t = mesh->soft_target ? mesh->soft_target : mesh->X0;
    h->soft_t.assign(t, t + h->N);
  }
  element_rest(h);
  build_pattern(h);
  *out = h;
  return 0;
}

void orc_destroy(orc_handle h) { delete h; }

int orc_material(int model, double lame1, double lame2, const double* Fv, double* psi, double* P,
                 double* dPdF) {
  material(model, lame1, lame2, Fv, psi, P, dPdF);
  return 0;
}

int orc_element_local(orc_handle h, const double* x, double* E, double* g, double* H) {
#pragma omp parallel for schedule(static)
  for (int e = 0; e < h->m; ++e)
    element_eval(h, e, x, E ? &E[e] : nullptr, g ? &g[(size_t)12 * e] : nullptr,
                 H ? &H[(size_t)144 * e] : nullptr);
  return 0;
}

int orc_energy(orc_handle h, const double* x, double* E) {
  *E = model_energy(h, x, nullptr);
  return 0;
}

int orc_gradient(orc_handle h, const double* x, double* g, int fix) {
  model_gradient(h, x, g, fix != 0, nullptr);
  return 0;
}

int64_t orc_hessian_nnz(orc_handle h) { return (int64_t)h->rowidx.size(); }

int orc_hessian_pattern(orc_handle h, int32_t* colptr, int32_t* rowidx) {
  std::copy(h->colptr.begin(), h->colptr.end(), colptr);
  std::copy(h->rowidx.begin(), h->rowidx.end(), rowidx);
  return 0;
}

int orc_hessian(orc_handle h, const double* x, double* vals, int fix) {
  model_hessian(h, x, vals, fix != 0, nullptr);
  return 0;
}

int orc_scatter_map(orc_handle h, int32_t* map) {
  // block slot = position of the block's (row 0, col 0) entry among the block-leading entries,
  // counted column-major: every stored 3x3 tile is one block.
  std::vector<int> lead_rank(h->rowidx.size(), -1);
  int nb = 0;
  for (int c = 0; c < h->N; c += 3)
    for (int q = h->colptr[c]; q < h->colptr[c + 1]; ++q)
      if (h->rowidx[q] % 3 == 0) lead_rank[q] = nb++;
  for (int e = 0; e < h->m; ++e)
    for (int p = 0; p < 10; ++p) {
      int li = kPairI[p], lj = kPairJ[p];
      int oi = 3 * h->T[4 * e + li], oj = 3 * h->T[4 * e + lj];
      int r = std::max(oi, oj), c = std::min(oi, oj);
      const int* beg = &h->rowidx[h->colptr[c]];
      const int* end = &h->rowidx[h->colptr[c + 1]];
      const int* it = std::lower_bound(beg, end, r);
      map[(size_t)e * 10 + p] = lead_rank[it - h->rowidx.data()];
    }
  return 0;
}

int orc_solve_static(orc_handle h, const orc_options* o, double* x, orc_report* rep) {
  h->cg_par = o->cg_parallel;
  if (h->cg_par) full_rows(h);
#ifdef _OPENMP
  int saved = omp_get_max_threads();
  if (o->threads > 0) omp_set_num_threads(o->threads);
#endif
  Problem P;
  P.h = h;
  P.x.assign(x, x + h->N);
  P.v.assign(h->N, 0.0);
  int rc = solve_full(h, P, o, rep);
  std::copy(P.x.begin(), P.x.end(), x);
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  return rc;
}

int orc_solve_dynamic(orc_handle h, const orc_options* o, double dt, double* x, double* v, orc_report* rep) {
  h->cg_par = o->cg_parallel;
  if (h->cg_par) full_rows(h);
#ifdef _OPENMP
  int saved = omp_get_max_threads();
  if (o->threads > 0) omp_set_num_threads(o->threads);
#endif
  Problem P;
  P.h = h;
  P.dynamic = true;
  P.dt = dt;
  P.x.assign(x, x + h->N);
  P.v.assign(v, v + h->N);
  int rc = solve_full(h, P, o, rep);
  std::copy(P.x.begin(), P.x.end(), x);
  std::copy(P.v.begin(), P.v.end(), v);
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  return rc;
}

int orc_linear_solve(orc_handle h, const orc_options* o, const double* x, const double* b, double* dx,
                     int32_t* lsresult, int64_t* iters) {
  h->cg_par = o->cg_parallel;
  if (h->cg_par) full_rows(h);
  std::vector<double> H(h->rowidx.size());
  model_hessian(h, x, H.data(), true, nullptr);
  std::vector<double> bb(b, b + h->N), xs(dx, dx + h->N);
  int reg = 0;
  int64_t it = 0;
  int r;
  if (o->ls_solver == 1)
    r = solve_cg(h, H, bb, xs, o->ls_tol_max_error, o->ls_num_max_iters, 10, o->cg_block_jacobi != 0, &reg, &it);
  else
    r = solve_ldlt(h, H, bb, xs, o->ls_tol_max_error, 10, &reg);
  std::copy(xs.begin(), xs.end(), dx);
  if (lsresult) *lsresult = r;
  if (iters) *iters = it;
  return 0;
}

int64_t orc_ldl_nnz(orc_handle h, int natural) {
  if (natural) {
    // analyse once with the identity ordering, report, then drop it
    orc_handle_s tmp;
    tmp.n = h->n; tmp.m = h->m; tmp.N = h->N; tmp.X0 = h->X0; tmp.T = h->T;
    tmp.colptr = h->colptr; tmp.rowidx = h->rowidx;
    for (int i = 0; i < tmp.n; ++i) tmp.X0[3 * i] = tmp.X0[3 * i + 1] = tmp.X0[3 * i + 2] = 0.0;
    ldl_analyse(&tmp);
    return tmp.ldl.Lp[tmp.N];
  }
  if (!h->ldl.analysed) ldl_analyse(h);
  return h->ldl.Lp[h->N];
}

int orc_set_staging(orc_handle h, int32_t count, const orc_stage_group* groups, int32_t num_stages,
                    const double* x_ini) {
  if (count < 0 || num_stages < 0 || (count > 0 && (!groups || !x_ini))) return -1;
  std::vector<orc_handle_s::Group> gs;
  int most = num_stages;
  for (int g = 0; g < count; ++g) {
    const orc_stage_group& G = groups[g];
    if (G.num_stages < 1 || G.num_nodes < 0 || (G.num_nodes > 0 && !G.nodes)) return -1;
    orc_handle_s::Group q;
    q.num_stages = G.num_stages;
    q.soft = G.soft ? 1 : 0;
    q.k0 = G.k_start;
    q.k1 = G.k_end;
    std::copy(G.move, G.move + 9, q.M);
    std::copy(G.shift, G.shift + 3, q.b);
    for (int k = 0; k < G.num_nodes; ++k) {
      const int i = G.nodes[k];
      if (i < 0 || i >= h->n) return -1;
      if (q.soft && (h->soft_k.empty() || h->soft_k[i] == 0.0)) return -1;
      q.nodes.push_back(i);
      for (int r = 0; r < 3; ++r) q.ini.push_back(x_ini[3 * i + r]);
    }
    most = std::max(most, G.num_stages);
    gs.push_back(std::move(q));
  }
  h->groups = std::move(gs);
  h->num_stages = most;
  h->stage = 0;
  return 0;
}

int orc_stage(orc_handle h) { return h->stage; }

int orc_set_soft(orc_handle h, const double* k, const double* t) {
  if (h->soft_k.empty() || !k || !t) return -1;
  for (int i = 0; i < h->n; ++i) {
    if (h->soft_k[i] == 0.0) continue;
    h->soft_k[i] = k[i];
    for (int c = 0; c < 3; ++c) h->soft_t[3 * i + c] = t[3 * i + c];
  }
  return 0;
}

int orc_last_log(orc_handle h, double* obj, double* opt, int32_t* bis, double* step, int32_t cap) {
  int n = std::min<int>((int)h->log_obj.size(), cap);
  for (int i = 0; i < n; ++i) {
    if (obj) obj[i] = h->log_obj[i];
    if (opt) opt[i] = h->log_opt[i];
    if (bis) bis[i] = h->log_bis[i];
    if (step) step[i] = h->log_step[i];
  }
  return (int)h->log_obj.size();
}

}  // extern "C"
