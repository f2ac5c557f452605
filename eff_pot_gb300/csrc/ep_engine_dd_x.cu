// ep_engine_dd_x.cu - double-float engine: poten and its X-pass dispatch.
#define EP_ENGINE_PARTS 2
#include "ep_engine_impl.cuh"
template int Engine<dfloat>::poten();
template int Engine<dfloat>::x_pass(int, bool);
template int Engine<dfloat>::x_attrs();
