// engine_fp64.cu -- the plain form: every per-particle field and pair
// interaction in FP64.
#include "engine_impl.cuh"

namespace dsph {
std::unique_ptr<EngineBase> make_engine_fp64(int device) {
    return std::unique_ptr<EngineBase>(new Engine<double>(device));
}
}  // namespace dsph
