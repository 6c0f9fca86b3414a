// FP64 instantiation: every operation of the step in double precision.
#include "engine_impl.cuh"
namespace qg {
EngineBase* make_engine_fp64() { return new Engine<double>(); }
}  // namespace qg
