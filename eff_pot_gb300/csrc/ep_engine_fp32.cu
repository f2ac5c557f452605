// ep_engine_fp32.cu - FP32 instantiation of the engine (bulk FP32 fields,
// FP64 reductions).
#include "ep_engine_impl.cuh"
template class Engine<float>;
template int Engine<float>::import_state<double>(const Engine<double>&);
