// engine_mixed.cu -- the mixed form: FP32 pair interactions, EOS and stress;
// FP64 positions, internal energy and conservation sums.
#include "engine_impl.cuh"

namespace dsph {
std::unique_ptr<EngineBase> make_engine_mixed(int device) {
    return std::unique_ptr<EngineBase>(new Engine<float>(device));
}
}  // namespace dsph
