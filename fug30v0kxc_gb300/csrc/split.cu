// split.cu -- FP32-bulk / FP64-background form (filled in below).
#include "common.cuh"
#include "engine.h"

int split_setup(Engine *E) { (void)E; vec_set_error("split form not built"); return VEC_ERR_ARG; }
int split_hydro(Engine *E) { (void)E; return VEC_ERR_ARG; }
int split_mag(Engine *E) { (void)E; return VEC_ERR_ARG; }
int split_bandj(Engine *E) { (void)E; return VEC_ERR_ARG; }
int split_refresh(Engine *E) { (void)E; return VEC_ERR_ARG; }
int split_ab3(Engine *E, int m) { (void)E; (void)m; return VEC_ERR_ARG; }
