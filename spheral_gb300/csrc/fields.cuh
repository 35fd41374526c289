// Field bank layout of libsphgpu: every per-node quantity is one device array
// (structure of arrays) in the cell-sorted node order of the current step.
#pragma once
#include "common.cuh"

namespace sph {

enum FieldId {
  // evolved / registered state
  F_X, F_Y, F_Z, F_VX, F_VY, F_VZ, F_MASS, F_RHO, F_EPS, F_HINV, F_P, F_CS, F_OMEGA,
  // derivatives read by the next step before they are recomputed (the
  // half-step predictor, the dt vote, the limited Q's DvDx copy)
  F_DXDT_X, F_DXDT_Y, F_DXDT_Z,
  F_DVDT_X, F_DVDT_Y, F_DVDT_Z,
  F_DRHODT, F_DEPSDT, F_DHDT, F_MAXQ,
  F_DVDX_XX, F_DVDX_XY, F_DVDX_XZ, F_DVDX_YX, F_DVDX_YY, F_DVDX_YZ, F_DVDX_ZX, F_DVDX_ZY, F_DVDX_ZZ,
  F_GRAV_X, F_GRAV_Y, F_GRAV_Z,
  // ASPH (tensor H) only: H as a symmetric tensor (xx xy xz yy yz zz), its
  // tensor DH/Dt and its largest eigenvalue (the dt node scale); F_HINV then
  // holds the smallest eigenvalue (1/h_max of the node: cell size and the
  // conservative neighbour pre-filter).  Permuted only in ASPH mode.
  F_HT_XX, F_HT_XY, F_HT_XZ, F_HT_YY, F_HT_YZ, F_HT_ZZ,
  F_DHDTT_XX, F_DHDTT_XY, F_DHDTT_XZ, F_DHDTT_YY, F_DHDTT_YZ, F_DHDTT_ZZ,
  F_HLMAX,
  F_NUM_CARRIED,
  // derivatives every evaluation rewrites (StateDerivatives of SPH,
  // SPHSmoothingScale, TreeGravity)
  F_GRADRHO_X = F_NUM_CARRIED, F_GRADRHO_Y, F_GRADRHO_Z,
  F_M_XX, F_M_XY, F_M_XZ, F_M_YX, F_M_YY, F_M_YZ, F_M_ZX, F_M_ZY, F_M_ZZ,
  F_RHOSUM, F_NORM, F_EFFQ, F_XSPHW, F_XSPHDV_X, F_XSPHDV_Y, F_XSPHDV_Z,
  F_HIDEAL, F_M0, F_M1_X, F_M1_Y, F_M1_Z, F_POT, F_DEPS_COMPAT,
  // the limited Q's copy of DvDx (state field ArtificialViscosityVelocityGradient,
  // refreshed from DvDx at every postStateUpdate)
  F_DVDXQ_XX, F_DVDXQ_XY, F_DVDXQ_XZ, F_DVDXQ_YX, F_DVDXQ_YY, F_DVDXQ_YZ, F_DVDXQ_ZX, F_DVDXQ_ZY, F_DVDXQ_ZZ,
  // ASPH only: tensor Hideal and the second moment of the neighbour distribution
  F_HIDEALT_XX, F_HIDEALT_XY, F_HIDEALT_XZ, F_HIDEALT_YY, F_HIDEALT_YZ, F_HIDEALT_ZZ,
  F_M2_XX, F_M2_XY, F_M2_XZ, F_M2_YY, F_M2_YZ, F_M2_ZZ,
  F_RAD0,          // ASPH radialOnly: |x| at the start of the step
  // CRKSPH only: the RK volume and the LinearOrder corrections (C_0..3, then
  // dC/dx, dC/dy, dC/dz with 4 entries each).  Permuted only in CRKSPH mode.
  F_VOL,
  F_RKC_0, F_RKC_1, F_RKC_2, F_RKC_3, F_RKC_4, F_RKC_5, F_RKC_6, F_RKC_7,
  F_RKC_8, F_RKC_9, F_RKC_10, F_RKC_11, F_RKC_12, F_RKC_13, F_RKC_14, F_RKC_15,
  F_NUM_PERMUTED,
  // beginning-of-step copies (not permuted: written after the sort)
  F_X0 = F_NUM_PERMUTED, F_Y0, F_Z0, F_VX0, F_VY0, F_VZ0, F_RHO0, F_EPS0, F_HINV0,
  F_HT0_XX, F_HT0_XY, F_HT0_XZ, F_HT0_YY, F_HT0_YZ, F_HT0_ZZ,
  F_VOL0,
  F_NUM_FIELDS
};

// Fields a permute moves: up to three index ranges [first, last) of Fields::f.
struct FieldRanges {
  int n;
  int first[3], last[3];
};

struct Fields {
  double* f[F_NUM_FIELDS];
};

// FP32 mirror of the pair-loop inputs (precision mode FP32).
struct Fields32 {
  float4* posh;     // (x - cell origin, y - ..., z - ..., hinv)
  float4* velm;     // (vx, vy, vz, m)
  float4* thermo;   // (rho, P/rho^2 * Omega^-1, cs, unused)
  uint32_t* cell;   // packed cell coordinates (10 bits per axis)
  float4* dvq;      // limited Q: DvDx of the Q as 3 float4 per node (xx xy xz yx | yy yz zx zy | zz - - -)
  float4* hten;     // ASPH: tensor H as 2 float4 per node (xx xy xz yy | yz zz det(H) lambda_max)
  float* vol;       // CRKSPH: RK volume
  float4* rkc;      // CRKSPH: LinearOrder corrections, 4 float4 per node (C | dC/dx | dC/dy | dC/dz)
};

}  // namespace sph
