// Kernels of one MF-LBM time step: AA-pattern collision + streaming
// (collide.cuh), the colour-gradient / CSF / wetting pipeline (gradient.cuh)
// and the boundary updates (boundary.cuh).
//
// This header is compiled twice: step_fast.cu (FMA contraction, the
// production flavour) and step_strict.cu (-fmad=false: every operation is
// the IEEE operation written in the source, in the reference's order, so the
// result is bit-identical to the reference's arithmetic).  MFLBM_NS names the
// flavour's namespace.
#pragma once
#ifndef MFLBM_NS
#error "define MFLBM_NS before including step_kernels.cuh"
#endif

#include "collide.cuh"
#include "gradient.cuh"
#include "boundary.cuh"
#include "batch.cuh"
