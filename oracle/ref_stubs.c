/* Link stubs for the ISPC kernels of the reference's "WENO6-optimized" interpolator
 * (sginterp2.cpp/sginterp3.cpp declare them extern "C").  ispc is not available and
 * that interpolator is off the flux-advection path, so calling any of these aborts.
 * Test infrastructure only (oracle/_ref). */
#include <stdio.h>
#include <stdlib.h>
#define STUB(name) void name(void) { fprintf(stderr, "reference ISPC kernel " #name " is not built\n"); abort(); }
STUB(ispc_interpolate_bilinear_double2)
STUB(ispc_interpolate_bilinear_float2)
STUB(ispc_interpolate_trilinear_double3)
STUB(ispc_interpolate_trilinear_float3)
STUB(ispc_interpolate_weno4_double2)
STUB(ispc_interpolate_weno4_double3)
STUB(ispc_interpolate_weno4_float2)
STUB(ispc_interpolate_weno4_float3)
STUB(ispc_interpolate_weno6_double2)
STUB(ispc_interpolate_weno6_double3)
STUB(ispc_interpolate_weno6_float2)
STUB(ispc_interpolate_weno6_float3)
