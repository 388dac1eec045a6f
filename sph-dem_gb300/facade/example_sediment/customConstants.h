/* Example SPH-DEM sedimentation case for the device façade (generated by
 * make_constants.py from the `sediment3d_small` workload: keep the two in step). */
#ifndef CUSTOMCONSTANTS_H
#define CUSTOMCONSTANTS_H

#include <cmath>

#define _3D_
#define NDIM 3
#define WENDLAND
#define VISC_MORRIS
#define VAR_H_CORRECTION
#define LIQ_DEM
#define LINEAR
#define NO_ANTICLUMPING

const double PI = 3.14159265;
const double RMIN[NDIM] = {0.0, 0.0, 0.0};
const double RMAX[NDIM] = {0.04, 0.04, 0.08};
const int PERIODIC[NDIM] = {1, 1, 0};
const int GHOST[2*NDIM] = {0, 0, 0, 0, 0, 0};
const double DENS_DROP[NDIM] = {0.0, 0.0, 0.0};
const double PSEP = 0.004;
const double HFAC = 1.5;
const double H = 0.006;
const double DENS = 1000.0;
const double REFD = 1000.0;
const double GAMMA = 7.0;
const double PRB = 89691.42857142857;
const double SPSOUND = 25.05673562138532;
const double VISCOSITY = 1e-06;
const double BFAC = 1.0;
const int OUTSTEP = 10;
const double MAXTIME = 5.986414282632196e-05 * OUTSTEP;
const int RESTART_EVERY_N_STEPS = 5;
#define TIME_OVERIDE 0
#define START_TIME 0
#define NSTEP_OVERIDE 0
#define START_NSTEP 0
const double DAMPTIME = 0.0;
const int MAX_NUM_PARTICLES_PER_CPU = 2456;
const int REINIT_DENS_EVERY_N_STEPS = 50000000;
const int REINIT_DENS_AT_N_STEPS = 50000000;
const double TIME_DROP_PARTICLE = 1e+30;
const double DEM_RADIUS = 0.002;
const double DEM_DENS = 2500.0;
const double DEM_K = 10000.0;
const double DEM_GAMMA = 0.27888707130151075;
const double DEM_VOL = 3.35103216e-08;
const double DEM_MIN_REDUCED_MASS = 0.5 * DEM_VOL * DEM_DENS;
const double LIQ_DEM_COUPLING_RADIUS = 0.012210953134688967;

#endif
