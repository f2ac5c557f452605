// ep_engine_dd.cu - double-float instantiation of the engine (FP64-class
// fields computed on the FP32 pipes, see ep_dd.cuh): the members outside the
// X passes, the FFT passes and the stencil marches, which are compiled in
// ep_engine_dd_x.cu, ep_engine_dd_fft.cu and ep_engine_dd_march.cu.
#define EP_ENGINE_PARTS 1
#include "ep_engine_impl.cuh"
template class Engine<dfloat>;
template int Engine<dfloat>::import_state<double>(const Engine<double>&);
template int Engine<dfloat>::import_state<float>(const Engine<float>&);
template int Engine<double>::import_state<dfloat>(const Engine<dfloat>&);
template int Engine<float>::import_state<dfloat>(const Engine<dfloat>&);
