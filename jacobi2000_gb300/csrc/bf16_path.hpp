// Tensor-core (tcgen05) BF16 forward path.
#pragma once

#include "runtime.hpp"

namespace jc {

class BF16Path {
   public:
    BF16Path(const Dims& d, const TensorMap& t, DeviceArena& arena);
    void forward(const Dims& d, const WeightsF32& w32, const Pack& p, int mode, cudaStream_t s);
};

}  // namespace jc
