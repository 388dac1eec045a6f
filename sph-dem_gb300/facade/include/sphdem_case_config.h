/*
 * The case's compile-time configuration (customConstants.h constants and
 * feature macros) as the run-time SphDemConfig of the C ABI.  Constants are
 * read under the same feature macros the reference's own headers read them
 * under, so any case that compiles with the reference compiles here.
 * Gravity, walls and freezing stay with the case's hooks.
 */
#ifndef SPHDEM_CASE_CONFIG_H
#define SPHDEM_CASE_CONFIG_H

#include <cstring>

#include "../../../include/sphdem.h"
#include "customConstants.h"
#include "demConstants.h"

#if !defined(WENDLAND)
#error "the device path implements the Wendland C2 kernel only (#define WENDLAND)"
#endif
/* Options of the reference's step (sph.h, sphIncompress.h/.cpp, dataLL.cpp)
 * that the device path does not implement: a case that defines one would
 * step differently, so it does not build.  Options that only add fields or
 * checks (CHECK_FOR_NAN, SAVE_VHALF, TEST_VISC, HACK_TO_SAVE_MEM,
 * DEFORMATION_MATRIX) and LIQ_DEM_CUSTOM_WALL_CONTACTS (without it the
 * reference looks for wall particles in the DEM lists, which hold DEM
 * particles only) do not change the step. */
#if defined(LUBRICATION) || defined(HERTZ) || defined(HERTZ_KUWABARA)
#error "DEM contact law not implemented by the device path (LINEAR only)"
#endif
#if defined(REINIT_DENS_MLS) || defined(SMOOTHED_VISC_VELOCITY) || defined(SMOOTHED_VISC_VELOCITY_MLS) || \
    defined(SMOOTHED_VISC_VELOCITY_HAT) || defined(SMOOTHING) || defined(SPH_SMOOTHING) || \
    defined(DIRECT_SMOOTHING) || defined(GRID_SMOOTHING) || defined(AVE_VELOCITY)
#error "MLS re-initialisation and velocity smoothing are not implemented by the device path"
#endif
#if defined(LIQ_DEM_SEPARATE_DRAGS) || defined(LIQ_DEM_SIMPLE_DRAG) || defined(LIQ_DEM_ERGUN_DRAG) || \
    defined(ERGUN) || defined(LIQ_DEM_LIFT) || defined(LIQ_DEM_ADDED_MASS) || defined(LIQ_DEM_ONE_WAY_COUPLE) || \
    defined(LIQ_DEM_TEST) || defined(LIQ_DEM_DENS_NORMAL) || defined(LIQ_DEM_DDDT_VER2) || \
    defined(LIQ_DEM_VARIABLE_TIMESTEP) || defined(_2D_DEM)
#error "SPH-DEM coupling variant not implemented by the device path (Di Felice drag, porosity-weighted continuity)"
#endif
#if defined(FIXED_DEM) || defined(NO_DEM_CONTACTS)
#error "FIXED_DEM / NO_DEM_CONTACTS are not implemented by the device path (freeze DEM particles in a hook)"
#endif
#if defined(SLK) || defined(VAR_H_CORRECTION2) || defined(MY_VAR_RES) || defined(DDENS_VARIANT) || \
    defined(DENS_DIFFUSE) || defined(DENS_DIFFUSE_PRESS) || defined(BACKGROUND_PRESSURE_FORCE) || \
    defined(INCL_THERM_ENERGY) || defined(HALF_COURANT)
#error "SPH step variant not implemented by the device path"
#endif
#if defined(VISC_CLEARY) || defined(MORRIS_SPH_BOUNDARY) || defined(SLIP_BOUNDARIES) || defined(RADIAL_BOUNDARY) || \
    defined(MODIFY_BFORCE_WITH_STILL_LEVEL) || defined(BORE_SOLITON)
#error "viscosity or boundary variant not implemented by the device path"
#endif

/* The two per-axis constants of the reference's ghost particles
 * (dataLL.cpp:648-683) that the device path does not implement: mirror
 * ghosts at GHOST[] walls, and a density offset DENS_DROP on crossing a
 * periodic boundary.  They are arrays, so the check runs at start-up:
 * the reason a case cannot run, or nullptr. */
inline const char *sphdem_case_unsupported() {
    for (int i = 0; i < 2 * NDIM; i++)
        if (GHOST[i] != 0) return "GHOST[] mirror boundaries are not implemented by the device path";
    for (int d = 0; d < NDIM; d++)
        if (PERIODIC[d] && DENS_DROP[d] != 0.0)
            return "DENS_DROP across a periodic boundary is not implemented by the device path";
    return nullptr;
}

inline SphDemConfig sphdem_case_config(int precision, bool fixed_dt) {
    SphDemConfig c;
    std::memset(&c, 0, sizeof c);
    c.ndim = NDIM;
    c.precision = precision;
#if defined(VISC_MORRIS)
    c.visc_model = SPHDEM_VISC_MORRIS;
#elif defined(VISC_MONAGHAN)
    c.visc_model = SPHDEM_VISC_MONAGHAN;
#elif defined(VISC_ARTIFICIAL)
    c.visc_model = SPHDEM_VISC_ARTIFICIAL;
    c.alpha_artificial = ALPHA_ARTIFICIAL;
#else
    c.visc_model = SPHDEM_VISC_NONE;
#endif
    c.flags = 0;
#ifdef CONST_H
    c.flags |= SPHDEM_F_CONST_H;
#endif
#ifdef NO_ANTICLUMPING
    c.flags |= SPHDEM_F_NO_ANTICLUMPING;
#endif
#ifdef VAR_H_CORRECTION
    c.flags |= SPHDEM_F_VAR_H_CORRECTION;
#endif
#ifdef LIQ_DEM
    c.flags |= SPHDEM_F_LIQ_DEM;
#endif
#ifdef CORRECTED_GRADIENT
    c.flags |= SPHDEM_F_CORRECTED_GRADIENT; /* both precisions; not with LIQ_DEM */
#endif
#if defined(LIQ_DEM) && defined(DEM_BLOCK)
    c.flags |= SPHDEM_F_DEM_BLOCK;
#endif
    if (fixed_dt) c.flags |= SPHDEM_F_FIXED_DT;
    c.pi = PI;
    for (int d = 0; d < NDIM; d++) {
        c.periodic[d] = PERIODIC[d];
        c.rmin[d] = RMIN[d];
        c.rmax[d] = RMAX[d];
        /* the processor domain of a single-rank setup: exact on periodic
         * axes, 25% margin on the others */
        const double ext = RMAX[d] - RMIN[d];
        c.domain_min[d] = PERIODIC[d] ? RMIN[d] : RMIN[d] - 0.25 * ext;
        c.domain_max[d] = PERIODIC[d] ? RMAX[d] : RMAX[d] + 0.25 * ext;
    }
    c.hfac = HFAC;
    c.psep = PSEP;
    c.h = H;
    c.dens = DENS;
    c.refd = REFD;
    c.gamma = GAMMA;
    c.prb = PRB;
    c.spsound = SPSOUND;
    c.viscosity = VISCOSITY;
    c.bfac = BFAC;
    c.maxdt = MAXTIME / OUTSTEP; /* run.cpp:87 */
    c.damptime = DAMPTIME;
    /* both constants are required, as sphIncompress.cpp:20 reads both */
    c.reinit_dens_every = REINIT_DENS_EVERY_N_STEPS;
    c.reinit_dens_at = REINIT_DENS_AT_N_STEPS;
#ifdef LIQ_DEM
    c.dem_radius = DEM_RADIUS;
    c.dem_dens = DEM_DENS;
    c.dem_k = DEM_K;
    c.dem_gamma = DEM_GAMMA;
    c.dem_search_radius = DEM_SEARCH_RADIUS;
    c.dem_vol = DEM_VOL;
    c.coupling_radius = LIQ_DEM_COUPLING_RADIUS;
#ifdef LINEAR
    c.dem_timestep = DEM_TIMESTEP;
#endif
    c.liq_dem_timestep = LIQ_DEM_TIMESTEP;
#endif
#if defined(LIQ_DEM) && !defined(FIXED_DEM) && !defined(NO_DEM_CONTACTS)
    c.time_drop_particle = TIME_DROP_PARTICLE; /* the DEM dt bound starts then (sphIncompress.cpp:133) */
#else
    c.time_drop_particle = 1e30;
#endif
    c.freeze_dem_until = -1.0; /* freezing is the case hooks' business */
    return c;
}

#endif
