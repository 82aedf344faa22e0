// Split-precision FP64 GEMM (placeholder until the tcgen05 engine lands).
#include "split.h"

namespace gbx {
struct SplitPlan {};
int create_split_plan(const std::vector<SplitProblem>&, int, SplitPlan** out) {
  *out = nullptr;
  return fail(GBX_EUNSUPPORTED, "split engine not built yet");
}
int run_split_plan(SplitPlan*, bool, cudaStream_t) { return fail(GBX_EUNSUPPORTED, "split engine not built yet"); }
void destroy_split_plan(SplitPlan* sp) { delete sp; }
double split_plan_bytes(const SplitPlan*) { return 0.0; }
}  // namespace gbx
