// ref_mcg_shim.cpp -- compiles the reference's own generated material code
// (include/PhySim/Utils/Auto/FEMVol_{CoNH,StVK}_{Energy,Gradient,Hessian}.mcg)
// into a small C-ABI library, exactly as MaterialModel_3Din3D_{CoNH,StVK}
// (include/PhySim/Physics/Elements/MaterialModels.h:166-299) includes it.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py into oracle/_ref/ when the
// reference sources are present; used only to generate and re-check the golden
// vectors under tests/golden/.  The .mcg sources are read from the reference
// tree at build time and are not part of this repository.
#include <cmath>

using std::log;
using std::pow;

extern "C" {

int ref_conh(double lame1, double lame2, const double* Fv, double* U, double* P, double* H) {
  {
#include "FEMVol_CoNH_Energy.mcg"
    *U = t31;
  }
  {
    double vgx[9];
#include "FEMVol_CoNH_Gradient.mcg"
    for (int i = 0; i < 9; ++i) P[i] = vgx[i];
  }
  {
    double mHx[9][9];
#include "FEMVol_CoNH_Hessian.mcg"
    for (int i = 0; i < 9; ++i)
      for (int j = 0; j < 9; ++j) H[9 * i + j] = mHx[i][j];
  }
  return 0;
}

int ref_stvk(double lame1, double lame2, const double* Fv, double* U, double* P, double* H) {
  {
#include "FEMVol_StVK_Energy.mcg"
    *U = t58;
  }
  {
    double vgx[9];
#include "FEMVol_StVK_Gradient.mcg"
    for (int i = 0; i < 9; ++i) P[i] = vgx[i];
  }
  {
    double mHx[9][9];
#include "FEMVol_StVK_Hessian.mcg"
    for (int i = 0; i < 9; ++i)
      for (int j = 0; j < 9; ++j) H[9 * i + j] = mHx[i][j];
  }
  return 0;
}

}  // extern "C"
