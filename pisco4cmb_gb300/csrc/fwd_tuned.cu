// fwd_tuned.cu -- TUNED forward (placeholder until the tuned kernel lands).
#include "internal.h"
namespace pisco {
bool tuned_supported(int, int, double) { return false; }
cudaError_t launch_forward_tuned(const FwdArgs&, int, cudaStream_t) { return cudaErrorNotSupported; }
}  // namespace pisco
