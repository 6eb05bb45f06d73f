// kg_lib.cu -- single translation unit of the device library (the kernels share the
// __constant__ run settings, so they are compiled together rather than with -rdc).
#include "kg_hydro.cu"
#include "kg_hydro32.cu"
#include "kg_tiles.cu"
#include "kg_dem.cu"

#include "kg_morpho.cu"
#include "kg_engine.cu"
#include "kg_noalloc.cu"
#include "kg_batch.cu"
