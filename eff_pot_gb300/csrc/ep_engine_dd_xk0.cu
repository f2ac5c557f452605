// ep_engine_dd_xk0.cu - double-float engine: the X-pass kernels (the general
// shared-memory engine on every half-line length).
#define EP_ENGINE_PARTS 16
#include "ep_engine_impl.cuh"
template int Engine<dfloat>::x_launch<0>(int, bool);
template int Engine<dfloat>::x_attrs_n2<0>();
