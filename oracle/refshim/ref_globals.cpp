/* Defines the reference's global variables (the role the reference's
 * src/main.cpp translation unit plays) for the host build in oracle/_ref. */
#include "externLib.h"
#include "solver_precision.h"
#include "preprocessor.h"
#include "Module_extern.h"
#include "Module.h"
#include "Fluid_singlephase_extern.h"
#include "Fluid_singlephase.h"
#include "Fluid_multiphase_extern.h"
#include "Fluid_multiphase.h"
