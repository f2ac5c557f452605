// ep_engine_dd_xk32.cu - double-float engine: the X-pass kernels on half-lines of 32 and 64 points
// (0: the general shared-memory engine).
#define EP_ENGINE_PARTS 16
#include "ep_engine_impl.cuh"
template int Engine<dfloat>::x_launch<32>(int, bool);
template int Engine<dfloat>::x_attrs_n2<32>();
template int Engine<dfloat>::x_launch<64>(int, bool);
template int Engine<dfloat>::x_attrs_n2<64>();
