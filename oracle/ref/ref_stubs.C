/*
 * Stand-ins for surface:: members that the reference's interpLib.C /
 * parallel.C reference but that live in reference files outside the
 * membrane-surface path (volume.C, get_regions.C, write_structures.C). The oracle driver never reaches them; each aborts.
 */
#include <stdio.h>
#include <stdlib.h>
#include "interp.h"

#define REF_STUB_ABORT(name) do { fprintf(stderr, "oracle: %s is outside the surface path\n", name); abort(); } while (0)

void surface::getRegions(int *, int) { REF_STUB_ABORT("surface::getRegions"); }
void surface::new_volume(double *, double *, double *, double *, double *) { REF_STUB_ABORT("surface::new_volume"); }
void surface::writeXYZSurface(const char *, const char *, surface *) { REF_STUB_ABORT("surface::writeXYZSurface"); }
void surface::writeXYZandPSFPeriodic(const char *) { REF_STUB_ABORT("surface::writeXYZandPSFPeriodic"); }
