// ep_engine_dd_fft.cu - double-float engine: the Y and Z transform passes.
#define EP_ENGINE_PARTS 4
#include "ep_engine_impl.cuh"
template int Engine<dfloat>::fft_y(dfloat2**, int, int);
template int Engine<dfloat>::zconv(const dfloat2* const*, dfloat2* const (*)[3], const dfloat* const (*)[3],
                                   const int*, int);
template int Engine<dfloat>::fft_attrs();
