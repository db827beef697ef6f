// Split-precision tensor-core contraction engine (sm_103a tcgen05).
// Placeholder until the kernel lands: requesting a split mode fails loudly.
#include "split_gemm.h"

namespace ccsd {

SplitEngine::SplitEngine(int nslices, cudaStream_t st) : nslices_(nslices), st_(st) {
    throw Error(-7, "split-precision engine not built yet");
}
SplitEngine::~SplitEngine() {}
void SplitEngine::gemm(int, int, int, double, const MatView &, const MatView &, double,
                       const OutView &, int, int) {}
int SplitEngine::error_status() { return 0; }
size_t SplitEngine::cached_bytes() const { return 0; }

}  // namespace ccsd
