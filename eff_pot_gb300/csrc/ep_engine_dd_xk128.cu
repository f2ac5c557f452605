// ep_engine_dd_xk128.cu - double-float engine: the X-pass kernels on half-lines of 128 points
// (0: the general shared-memory engine).
#define EP_ENGINE_PARTS 16
#include "ep_engine_impl.cuh"
template int Engine<dfloat>::x_launch<128>(int, bool);
template int Engine<dfloat>::x_attrs_n2<128>();
