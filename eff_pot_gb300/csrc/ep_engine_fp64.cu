// ep_engine_fp64.cu - FP64 instantiation of the engine (the drop-in path).
#include "ep_engine_impl.cuh"
template class Engine<double>;
template int Engine<double>::import_state<float>(const Engine<float>&);
