// Mixed-precision instantiation: FP32 transforms, products and update;
// FP64 tridiagonal solves and diagnostics.
#include "engine_impl.cuh"
namespace qg {
EngineBase* make_engine_fp32() { return new Engine<float>(); }
}  // namespace qg
