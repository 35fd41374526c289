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
  F_NUM_PERMUTED,
  // beginning-of-step copies (not permuted: written after the sort)
  F_X0 = F_NUM_PERMUTED, F_Y0, F_Z0, F_VX0, F_VY0, F_VZ0, F_RHO0, F_EPS0, F_HINV0,
  F_NUM_FIELDS
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
};

}  // namespace sph
