#include "bf16_path.hpp"

namespace jc {

BF16Path::BF16Path(const Dims&, const TensorMap&, DeviceArena&) {
    throw Error(JC_BAD_ARGUMENT, "the BF16 path is not available in this build");
}

void BF16Path::forward(const Dims&, const WeightsF32&, const Pack&, int, cudaStream_t) {}

}  // namespace jc
