// Test-only C shim over the product's Newton state machine (physim_gb300/csrc/newton_control.h),
// so its transitions can be driven on the host against the CPU oracle.
#include "newton_control.h"

extern "C" {
int ctl_sizes(int* out) {
  out[0] = (int)sizeof(phx::NState);
  out[1] = (int)sizeof(phx::DevOpts);
  return 0;
}
void ctl_advance_c(phx::NState* s, const phx::DevOpts* o) { phx::ctl_advance(*s, *o); }
}
