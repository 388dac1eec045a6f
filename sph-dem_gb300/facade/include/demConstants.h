/*
 * DEM constants derived from the case constants for LIQ_DEM cases, with the
 * reference's definitions (demConstants.h): the DEM search radius, the
 * contact and the liquid-coupling time step bounds.
 */
#ifndef DEMCONSTANTS_H
#define DEMCONSTANTS_H

#include <cmath>

#include "customConstants.h"

#ifdef LIQ_DEM
#ifdef LINEAR
const double DEM_TIMESTEP =
    (1.0 / 50.0) * PI / std::sqrt(DEM_K / DEM_MIN_REDUCED_MASS - std::pow(0.5 * DEM_GAMMA / DEM_MIN_REDUCED_MASS, 2));
#endif
const double DEM_SEARCH_RADIUS = 1.0 * DEM_RADIUS;
const double LIQ_DEM_TIMESTEP = (1.0 / 5.0) * DEM_VOL * DEM_DENS / (6.0 * PI * VISCOSITY * DENS * DEM_RADIUS);
#endif

#endif
