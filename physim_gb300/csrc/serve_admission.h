// serve_admission.h -- admission of serving requests by free slots and a device-memory budget.
//
// The serving loop (phx_server_* in engine.cu) admits queued requests at Newton-round
// boundaries.  A request needs a slot and, when its instance is not yet on the device,
// the device bytes of that instance; the instances a server created stay resident while
// idle (their mesh, pattern and last solution kept for warm re-solves) and their bytes
// count against its budget.  When a request does not fit, the least recently used idle
// instances are evicted (their positions kept on the host) until it does.  Plain C++, so
// the host tests drive the same decisions the server takes.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <vector>

namespace phx {

enum AdmitVerdict : int32_t {
  ADMIT = 0,        // fits now
  WAIT_SLOTS = 1,   // every slot is taken: retry after a request finishes
  WAIT_MEMORY = 2,  // the budget is taken by active requests: retry after one finishes
  EVICT = 3,        // fits once the planned idle instances are evicted
  NEVER = 4,        // larger than the whole budget: refused
};

// One resident instance the server may evict: its device bytes, the server tick of its
// last request, and whether it is idle (not queued, not active).
struct Resident {
  int64_t bytes;
  uint64_t last_used;
  bool idle;
};

// need: device bytes the request adds (0 when its instance is resident and counted).
// On EVICT, `plan` holds the indices into `res` to evict, least recently used first.
inline int32_t admit_decision(int active, int max_slots, int64_t in_use, int64_t budget, int64_t need,
                              const std::vector<Resident>& res, std::vector<int>* plan) {
  if (plan) plan->clear();
  if (need > budget) return NEVER;
  if (active >= max_slots) return WAIT_SLOTS;
  if (in_use + need <= budget) return ADMIT;
  std::vector<int> idx;
  for (int i = 0; i < (int)res.size(); ++i)
    if (res[i].idle && res[i].bytes > 0) idx.push_back(i);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return res[a].last_used < res[b].last_used; });
  int64_t freed = 0;
  std::vector<int> chosen;
  for (int i : idx) {
    if (in_use - freed + need <= budget) break;
    freed += res[i].bytes;
    chosen.push_back(i);
  }
  if (in_use - freed + need > budget) return WAIT_MEMORY;
  if (plan) *plan = chosen;
  return EVICT;
}

}  // namespace phx
