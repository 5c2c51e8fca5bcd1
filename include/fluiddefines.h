/*
 * fluiddefines.h - defaults of the FluidSystem interface.
 *
 * Same macro names and values as NCCA/libfluid's common/include/fluiddefines.h
 * (lines 4-25), which fluidsystem.h's default arguments and callers use.
 */
#ifndef FLUIDDEFINES_H
#define FLUIDDEFINES_H

#include <limits.h>

#define DEFAULT_TIMESTEP 0.01f
#define DEFAULT_REST_DENSITY 1.0f
#define DEFAULT_GAS_CONSTANT 1.0f
#define MAX_BOUNDING_PLANES 8
#define NULL_HASH UINT_MAX
#ifndef CUDART_PI_F
#define CUDART_PI_F 3.141592654f
#endif
#define DEFAULT_SURFACE_TENSION_FORCE 1.0f
#define DEFAULT_VISCOSITY_FORCE 0.1f
#define DEFAULT_ADHESION_FORCE 1.0f
#define DEFAULT_BOUNDARY_DENSITY 2600

#endif /* FLUIDDEFINES_H */
