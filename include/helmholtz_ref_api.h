/*
 * helmholtz_ref_api.h -- drop-in replacements for the reference's library
 * entry points (moorhsum/Helmholtz-3D-torrone), with the reference's own
 * signatures and C++ linkage, so a driver compiled with g++ against the
 * reference headers links against libhzgb300.so unchanged.
 *
 * The reference compiles its C sources as C++ (Makefile:1-3) and its
 * headers carry no extern "C", so these names are C++-mangled exactly like
 * the reference's objects.  Buffers are host memory owned by the caller,
 * as in the reference; the work runs on the current CUDA device.  Unlike
 * the reference, failures return a negative HZ_ERR_* status (message from
 * hz_last_error()) instead of calling exit(0).
 */
#ifndef HELMHOLTZ_REF_API_H
#define HELMHOLTZ_REF_API_H

#include "helmholtz_gb300.h"

/* distance_application3D.h:12 -- WENO (weno_mode 3 or 5) Godunov-upwinded
 * gradient of the distance grid at every node, distance_application3D.c:56-140.
 * Grids are the reference's ragged [SIZE][SIZE][SIZE] arrays, SIZE = N+1. */
HZ_API int ASSIGN_GRADIENT(int N, double H, double ***dist, double ***graddx, double ***graddy,
                           double ***graddz, int weno_mode);

/* Whole-grid form of the BothCurvs loop of large3Dexample2.c:446-455
 * (BothCurvs: distance_application3D.c:35-53, distance_application3D.h:11):
 * mean and Gaussian curvature at every node.  New entry point; the
 * reference calls BothCurvs once per node. */
HZ_API int ASSIGN_CURVATURES(int N, double H, double ***dist, double ***mcurv, double ***gcurv);

/* BICGSTAB.h:15 -- complex BiCG on a dense caller-owned matrix
 * (BICGSTAB.c:5-339): tolerance DEFAULTACC = 1e-7, at most 1000 iterations. */
HZ_API int CompBiCG(int size, double *density, double *densityimg, double **Kernel, double **Kernelimg,
                    double *b, double *bimg);

/* BICGSTAB.h:16-17 -- the OpenMP variant (BICGSTAB.c:344-765), at most 2000
 * iterations; chunk is accepted and ignored. */
HZ_API int omp_CompBiCG(int size, double *density, double *densityimg, double **Kernel, double **Kernelimg,
                        double *b, double *bimg, int chunk);

#endif
