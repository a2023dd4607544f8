/* Forced-include header for the FP64 oracle build of the reference (oracle/ref.mk, target fp64).
 * It pulls in the reference's own Utils/BGTypes.h first (include guard set), then switches the
 * BGFLOAT macro from float to double, which is the one-line change the reference documents at
 * Utils/BGTypes.h:17-23.  The reference tree itself is never modified. */
#include "BGTypes.h"
#undef SINGLEPRECISION
#undef BGFLOAT
#define DOUBLEPRECISION
#define BGFLOAT double
