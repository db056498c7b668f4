// ORACLE - test infrastructure only.  Compiles the reference's own uniform kernels, from
// src/tgv3d_uniform.cu where it lies in the reference checkout, into a cubin (device code only) that
// oracle/refrun.cpp loads on the GPU to pin the CPU oracle and to check the engine against the
// reference bit for bit where the arithmetic allows.  Nothing of the reference is copied: the file
// is included from its own location by the build recipe (oracle/build.py, -I <reference>/src).
#define main jp_ref_main_uniform
#include "tgv3d_uniform.cu"
