// admission_shim.cpp -- C entry point over serve_admission.h for the host tests.
#include <vector>

#include "serve_admission.h"

extern "C" int adm_decide(int active, int max_slots, long long in_use, long long budget, long long need, int count,
                          const long long* bytes, const unsigned long long* last_used, const int* idle, int* plan,
                          int* plan_len) {
  std::vector<phx::Resident> res(count);
  for (int i = 0; i < count; ++i) res[i] = {bytes[i], last_used[i], idle[i] != 0};
  std::vector<int> p;
  const int v = phx::admit_decision(active, max_slots, in_use, budget, need, res, &p);
  *plan_len = (int)p.size();
  for (int i = 0; i < (int)p.size(); ++i) plan[i] = p[i];
  return v;
}
