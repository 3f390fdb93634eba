// project_tc.cu -- tensor-core form of the fused projection (placeholder until
// the tcgen05 kernel lands): reports no supported shapes.
#include "engine.h"

namespace opsec {
bool project_tc_supported(const ProjectArgs&) { return false; }
size_t project_tc_work_bytes(const ProjectArgs&) { return 0; }
void launch_project_tc(const ProjectArgs&, cudaStream_t, long long*) {
    fail(OPSEC_ERR_STATE, "tensor-core projection unavailable");
}
}  // namespace opsec
