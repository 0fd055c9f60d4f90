// Tree-contact worlds (floating-base trees on a plane with a Newton or PGS
// constraint solve).  Placeholder dispatch until the kernel lands: such
// worlds are rejected at step time with a clear error.
#include "runtime.h"

extern "C" int newt_tc_step(newt_gpu_ctx* ctx, HostGroup* g, int n_steps, int fused) {
  (void)g; (void)n_steps; (void)fused;
  ctx->err = "tree-contact worlds are not supported by this build";
  return NEWT_E_INVALID;
}
