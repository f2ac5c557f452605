// ep_engine_dd_march.cu - double-float engine: the stencil marches
// (predictor, corrector, Runge-Kutta stage, first-derivative marches).
#define EP_ENGINE_PARTS 8
#include "ep_engine_impl.cuh"
template int Engine<dfloat>::d1march(int, const dfloat*, const dfloat*, dfloat*, dfloat*, dfloat*);
template int Engine<dfloat>::launch_march(const void*, dim3, dim3, size_t, void**, const char*, int);
template int Engine<dfloat>::lap_predict(double);
template int Engine<dfloat>::lap_correct(double, bool);
template int Engine<dfloat>::steppc_update(double, cudaGraphExec_t, cudaGraphNode_t, cudaGraphNode_t);
template int Engine<dfloat>::rk_stage(int, double);
template int Engine<dfloat>::march_setup();
