// ORACLE - test infrastructure only.  Compiles the reference's own AMR kernels, from
// src/tgv3d_amr.cu where it lies in the reference checkout, into a cubin (device code only) for
// oracle/refrun.cpp.  CUDA 13's Thrust (CCCL 3) no longer has thrust::identity, which the reference's
// host code names; oracle/thrust_identity_shim.h supplies it so the unmodified file compiles.
#define main jp_ref_main_amr
#include "tgv3d_amr.cu"
