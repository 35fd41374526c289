/*
 * sphgpu.h -- C ABI of the GB300-native SPH hydro package (libsphgpu.so).
 *
 * The library replaces, on one GPU, the ideal-gas SPH hot path of Spheral:
 * the connectivity build, the density sum, the SPH pair loop with the
 * TableKernel, Monaghan-Gingold viscosity and compatible-energy pair work,
 * the SPH smoothing-scale (IdealH) update, the TreeGravity walk and the
 * CheapSynchronousRK2 state update.  All particle state stays resident on the
 * device between calls; host arrays cross the boundary only in
 * sphgpu_set_particles / sphgpu_get_field / sphgpu_set_field.
 *
 * Conventions
 *  - Every entry point returns an int status: SPHGPU_OK (0) or one of the
 *    SPHGPU_E_* codes below; sphgpu_last_error() gives a readable message.
 *    No C++ exception crosses this boundary (the reference raises
 *    VERIFYError, src/Utilities/DBC.hh:175-183; a C++ shim maps non-zero
 *    codes back to that).
 *  - Arrays are host pointers in the reference's FieldList layouts:
 *    Vector = 3 doubles per node, SymTensor = 6 doubles per node in the order
 *    (xx, xy, xz, yy, yz, zz), Tensor = 9 doubles row-major (xx, xy, xz, yx,
 *    ..., zz).  Node order is the caller's order and is preserved.
 *  - Calls on one handle are synchronous on a library-owned CUDA stream and
 *    must not overlap (the reference calls packages from one host thread,
 *    src/Integrator/Integrator.cc:219-230).
 *
 * Reference interfaces each entry point replaces are cited as
 * path:line inside the llnl/spheral source tree.
 */
#ifndef SPHGPU_H
#define SPHGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SPHGPU_OK 0
#define SPHGPU_E_CUDA 1         /* a CUDA runtime call failed                        */
#define SPHGPU_E_ARG 2          /* bad argument (null pointer, size, unknown name)   */
#define SPHGPU_E_UNSUPPORTED 3  /* input outside the supported path (e.g. non-isotropic H) */
#define SPHGPU_E_OVERFLOW 4     /* a capacity limit was exceeded                     */
#define SPHGPU_E_NAN 5          /* non-finite or non-physical state detected         */
#define SPHGPU_E_TIMEOUT 6      /* a bounded device wait ran out                     */
#define SPHGPU_E_STATE 7        /* call out of order (e.g. step before set_particles) */

#define SPHGPU_PRECISION_FP64 0   /* every pair sum in FP64                               */
#define SPHGPU_PRECISION_FP32 1   /* FP32 pair loop on cell-relative positions, compensated sums */
#define SPHGPU_PRECISION_FP32_PLAIN 2  /* the same FP32 sweeps with plain (uncompensated) FP32 sums: the
                                          "FP32-relative" mode of the throughput sweep, kept to measure
                                          what compensation costs and buys (momentum drifts at ~1e-7) */

#define SPHGPU_BOUNDARY_PERIODIC 0
#define SPHGPU_BOUNDARY_REFLECTING 1

#define SPHGPU_DENSITY_RIGOROUS_SUM 0   /* MassDensityType::RigorousSumDensity */
#define SPHGPU_DENSITY_INTEGRATE 1      /* MassDensityType::IntegrateDensity   */

#define SPHGPU_VISCOSITY_MONAGHAN_GINGOLD 0          /* MonaghanGingoldViscosity        */
#define SPHGPU_VISCOSITY_LIMITED_MONAGHAN_GINGOLD 1  /* LimitedMonaghanGingoldViscosity (the SPH() factory default) */

/* HEvolutionType (src/SmoothingScale/SmoothingScaleBase.hh:26-30) */
#define SPHGPU_H_IDEAL 0       /* IdealH: the full update replaces H by Hideal (ReplaceBoundedState) */
#define SPHGPU_H_INTEGRATE 1   /* IntegrateH: H += dt DHDt, bounded (IncrementBoundedState)        */
#define SPHGPU_H_FIXED 2       /* FixedH: H never changes (FixedSmoothingScale)                    */

#define SPHGPU_SMOOTHING_SPH 0           /* SPHSmoothingScale: isotropic H = I/h                  */
#define SPHGPU_SMOOTHING_ASPH_CLASSIC 1  /* ASPHClassicSmoothingScale (SPH(..., ASPH="CLASSIC")):
                                            symmetric-tensor H                                  */
#define SPHGPU_SMOOTHING_ASPH 2          /* ASPHSmoothingScale (SPH(..., ASPH=True)) with fix_shape or
                                            radial_only: H integrated with DH/Dt in the step
                                            (IncrementASPHHtensor) and reset from the zeroth moment
                                            at its end; the Voronoi-shaped form is not built      */

/* Base kernel of the TableKernel (cfg.kernel, cfg.kernel_order). */
#define SPHGPU_KERNEL_BSPLINE 0   /* BSplineKernel (cubic, extent 2), the default            */
#define SPHGPU_KERNEL_NBSPLINE 1  /* NBSplineKernel(order), order 2..9, extent (order+1)/2    */
#define SPHGPU_KERNEL_WENDLAND_C2 2  /* WendlandC2Kernel (3-D form), extent 1                */
#define SPHGPU_KERNEL_WENDLAND_C4 3  /* WendlandC4Kernel (3-D form), extent 1                */

/* Hydro package (cfg.hydro). */
#define SPHGPU_HYDRO_SPH 0     /* SPH (src/SPH/SPH.cc)                                              */
#define SPHGPU_HYDRO_CRKSPH 1  /* CRKSPH with LinearOrder reproducing kernels (src/CRKSPH/CRKSPH.cc,
                                  RKCorrections): both precision modes, isotropic H, no grad-h    */

/* RK volume weighting of CRKSPH (cfg.rk_volume, RKVolumeType of
 * src/RK/RKCorrectionParams.hh; RKVoronoiVolume and RKHullVolume need a
 * tessellation and are not built). */
#define SPHGPU_RK_VOLUME_MASS_OVER_DENSITY 0  /* RKMassOverDensity: V = m / rho             */
#define SPHGPU_RK_VOLUME_SUM 1                /* RKSumVolume: V = 1 / sum_j W_ij            */
#define SPHGPU_RK_VOLUME_H 4                  /* HVolume: V = (pi / 6) / det(nPerh H)       */

typedef struct sphgpu_ctx* sphgpu_handle;

/* Package, artificial-viscosity, integrator and gravity settings.  Field
 * meanings follow the reference constructors:
 *   SPH(...) factory             src/SPH/SPHHydros.py:9-33
 *   SPH<Dim<3>> constructor      src/SPH/SPH.cc:43-79
 *   MonaghanGingoldViscosity     src/ArtificialViscosity/MonaghanGingoldViscosity.cc:25-37
 *   ArtificialViscosityHandle    src/ArtificialViscosity/ArtificialViscosityHandle.cc:36-54 (epsilon2)
 *   Integrator dtMin/dtMax/dtGrowth  src/Integrator/Integrator.cc:43-47
 *   OctTreeGravity(G, softeningLength, opening, ftimestep) src/Gravity/TreeGravity.cc:88-115
 *   LimitedMonaghanGingoldViscosity(Cl, Cq, kernel, linearInExpansion,
 *     quadraticInExpansion, etaCritFrac, etaFoldFrac)
 *                                src/ArtificialViscosity/LimitedMonaghanGingoldViscosity.cc:39-53,
 *                                defaults src/PYB11/ArtificialViscosity/LimitedMonaghanGingoldViscosity.py:31-32
 *   ASPHClassicSmoothingScale(HUpdate, W, fixShape, radialOnly)
 *                                src/SmoothingScale/ASPHClassicSmoothingScale.cc:34-46 (radialOnly
 *                                with the default ASPHRadialFunctor, about the origin) */
typedef struct sphgpu_config {
  int num_table_points;             /* TableKernel(BSplineKernel3d(), numPoints)           */
  double cfl;
  int use_velocity_magnitude_for_dt;
  int compatible_energy;            /* compatibleEnergyEvolution                           */
  int gradh_correction;
  int xsph;
  int correct_velocity_gradient;
  int sum_mass_density_over_all_nodelists;
  int density_update;               /* SPHGPU_DENSITY_*                                    */
  double eps_tensile, n_tensile;
  double Cl, Cq, eps2;
  int linear_in_expansion, quadratic_in_expansion;
  double dt_min, dt_max, dt_growth, last_dt, time;
  int gravity;
  double G, softening, opening, ftimestep;
  int precision;                    /* SPHGPU_PRECISION_*                                  */
  int device;                       /* CUDA device ordinal                                 */
  int viscosity;                    /* SPHGPU_VISCOSITY_*                                  */
  double eta_crit_frac, eta_fold_frac;  /* limited Q: full Q below etaCritFrac/nPerh      */
  int smoothing_scale;              /* SPHGPU_SMOOTHING_*                                  */
  int fix_shape;                    /* ASPH fixShape: Hideal keeps the shape of H          */
  int h_update;                     /* SPHGPU_H_* (the SPH() HUpdate argument)             */
  int evolve_total_energy;          /* evolveTotalEnergy (exclusive with compatible_energy) */
  int radial_only;                  /* ASPH radialOnly: H reshaped radially about the origin */
  int hydro;                        /* SPHGPU_HYDRO_* (CRKSPH(...) factory: CRKSPHHydros.py:9-110) */
  int rk_volume;                    /* SPHGPU_RK_VOLUME_* (SpheralController volumeType)    */
  int kernel;                       /* SPHGPU_KERNEL_*: base kernel of the built-in table    */
  int kernel_order;                 /* NBSplineKernel order                                  */
} sphgpu_config;

/* Fill *cfg with the reference defaults of the SPH() factory (cfl 0.25,
 * compatible energy, grad-h on, XSPH off in this path, corrected velocity
 * gradient, RigorousSumDensity), MG Cl = Cq = 1, epsilon2 = 1e-2, FP64.
 * Replaces: the keyword defaults of src/SPH/SPHHydros.py:9-33. */
void sphgpu_default_config(sphgpu_config* cfg);

/* Create a context on cfg->device.  Replaces: SPH<Dim<3>>::SPH
 * (src/SPH/SPH.cc:43-79) together with its Q sub-package and the
 * SPHSmoothingScale post sub-package (src/SPH/SPHHydros.py:125-140). */
int sphgpu_create(const sphgpu_config* cfg, sphgpu_handle* out);
int sphgpu_destroy(sphgpu_handle h);
const char* sphgpu_last_error(sphgpu_handle h);

/* Build the cubic B-spline TableKernel on the host into caller buffers.
 * w, grad, grad2: 3*(n1+1) coefficients each (n1 = (numPoints|1 - 1)/2 - 1);
 * nperh, wsum: 2*numPoints values each (Hermite knot values then slopes);
 * meta[9] = {n1, xstep, numPoints, nperh_xmin, nperh_xmax, wsum_xmin,
 * wsum_xmax, minNperh, maxNperh}.
 * Replaces: TableKernel<Dim<3>>::TableKernel (src/Kernel/TableKernel.cc:169-209). */
int sphgpu_build_bspline_table(int num_points, double* w, double* grad, double* grad2,
                               double* nperh, double* wsum, double* meta);

/* The TableKernel of a base kernel (kernel = SPHGPU_KERNEL_*, order for
 * NBSplineKernel): the layouts of sphgpu_build_bspline_table, and meta[9]
 * receives the kernel extent (meta has 10 entries).
 * Replaces: TableKernel<Dim<3>>::TableKernel(NBSplineKernel(order), numPoints)
 * (src/Kernel/TableKernel.cc:169-209, src/Kernel/NBSplineKernel.cc:20-118). */
int sphgpu_build_kernel_table(int kernel, int order, int num_points, double* w, double* grad, double* grad2,
                              double* nperh, double* wsum, double* meta);

/* Install a kernel table (the product of a reference TableKernel or of
 * sphgpu_build_bspline_table; same layouts).  Replaces: the TableKernelView
 * handed to the pair loops (src/Kernel/TableKernelView.hh:17-81). */
int sphgpu_set_kernel_table(sphgpu_handle h, const double* w, const double* grad, const double* grad2,
                            const double* nperh, const double* wsum, const double* meta);

/* Per-NodeList parameters.  Replaces: FluidNodeList(name, eos, ..., hmin,
 * hmax, hminratio, nPerh, maxNumNeighbors, rhoMin, rhoMax)
 * (src/NodeList/FluidNodeLists.py:15-47) + GammaLawGas(gamma)
 * (src/Material/GammaLawGas.cc:185-243). */
int sphgpu_set_nodelist(sphgpu_handle h, int nodelist, double nPerh, double hmin, double hmax,
                        double rhoMin, double rhoMax, double gamma);

/* NodeList::hminratio (default 0.1): the ASPH smoothing scale keeps every
 * eigenvalue of 1/h within 1/hminratio of the smallest.  Replaces: the
 * hminratio argument of FluidNodeList (src/NodeList/FluidNodeLists.py:21)
 * as read by ASPHClassicSmoothingScale.cc:219-288. */
int sphgpu_set_nodelist_hminratio(sphgpu_handle h, int nodelist, double hminratio);

/* Axis-aligned boundary.  type SPHGPU_BOUNDARY_PERIODIC: planes at lo and hi.
 * type SPHGPU_BOUNDARY_REFLECTING: one wall, at lo with normal +axis
 * (wall_high = 0) or at hi with normal -axis (wall_high = 1).
 * Replaces: PeriodicBoundary(plane1, plane2) (src/Boundary/PeriodicBoundary.cc:54-63)
 * and ReflectingBoundary(plane) (src/Boundary/ReflectingBoundary.cc:140-166),
 * whose ghost nodes become implicit periodic/mirror images. */
int sphgpu_add_boundary(sphgpu_handle h, int type, int axis, double lo, double hi, int wall_high);

/* Upload n internal nodes (host arrays, caller order).  H (xx xy xz yy yz zz
 * per node) must be isotropic (H = I/h, the form SPHSmoothingScale
 * maintains) unless the ASPH smoothing scale is selected, in which case it
 * must be symmetric positive definite; otherwise SPHGPU_E_UNSUPPORTED /
 * SPHGPU_E_NAN.  nodelist may be NULL (all zero).
 * Replaces: the registered state FieldLists of SPHBase::registerState
 * (src/SPH/SPHBase.cc:203-263). */
int sphgpu_set_particles(sphgpu_handle h, long n, const double* pos, const double* vel, const double* mass,
                         const double* rho, const double* eps, const double* H, const int* nodelist);

/* Pressure, sound speed and grad-h correction of the current state.
 * Replaces: SPHBase::initializeProblemStartupDependencies (src/SPH/SPHBase.cc:152-197). */
int sphgpu_initialize(sphgpu_handle h);

/* Rebuild the neighbour lists from the current positions and H.
 * Replaces: ConnectivityMap::computeConnectivity (src/Neighbor/ConnectivityMap.cc:747-1029)
 * after Integrator::setGhostNodes (src/Integrator/Integrator.cc:372-540). */
int sphgpu_connectivity(sphgpu_handle h);

/* Replace the mass density by the SPH sum.  Replaces: computeSPHSumMassDensity
 * (src/SPH/computeSPHSumMassDensity.cc:15-87) via SPHBase::preStepInitialize. */
int sphgpu_sum_density(sphgpu_handle h);

/* Grad-h correction.  Replaces: computeSPHOmegaGradhCorrection
 * (src/SPH/computeSPHOmegaGradhCorrection.cc:15-116) via SPHBase::postStateUpdate. */
int sphgpu_gradh(sphgpu_handle h);

/* Evaluate all derivatives on the current state with the current neighbour
 * lists.  Replaces: SPH::evaluateDerivatives (src/SPH/SPH.cc:143-555),
 * SPHSmoothingScale::evaluateDerivatives (src/SmoothingScale/SPHSmoothingScale.cc:101-275),
 * TreeGravity::evaluateDerivatives (src/Gravity/TreeGravity.cc:146-331) when
 * gravity is on, and SPHBase::finalizeDerivatives (src/SPH/SPHBase.cc:499-521). */
int sphgpu_evaluate_derivatives(sphgpu_handle h);

/* Time-step vote (already multiplied by cfl).  reason: 0 sound speed,
 * 1 artificial viscosity, 2 velocity divergence, 3 acceleration,
 * 4 velocity magnitude, 5 pairwise velocity difference, 6 gravity.
 * Replaces: GenericHydro::dt (src/Physics/GenericHydro.cc:113-381) and
 * TreeGravity::dt (src/Gravity/TreeGravity.cc:484-520). */
int sphgpu_dt(sphgpu_handle h, double* dt, int* reason);

/* One CheapSynchronousRK2 step bounded by max_time; *dt_out gets the step.
 * Replaces: Integrator::step (src/Integrator/Integrator.cc:67-110) ->
 * CheapSynchronousRK2::step (src/Integrator/CheapSynchronousRK2.cc:40-132). */
int sphgpu_step(sphgpu_handle h, double max_time, double* dt_out);

/* nsteps calls of sphgpu_step (stops early at max_time). */
int sphgpu_advance(sphgpu_handle h, int nsteps, double max_time);

/* Batched ensemble: nsteps CheapSynchronousRK2 steps on each of nboxes
 * independent handles (separate problems, e.g. turbulent boxes of uneven
 * sizes).  Handles are spread over nthreads host threads (0: one per
 * hardware thread), largest particle count first onto the least-loaded
 * thread; every handle runs on its own stream, so the GPU overlaps the
 * kernels of different boxes and small boxes do not leave it idle.  Each
 * box's result is bitwise that of sphgpu_advance on the handle alone.  The
 * handles must be distinct and not used by other threads meanwhile.  On a
 * failure the remaining boxes stop at their next step boundary, *failed (if
 * not NULL) receives the index of the first failing handle (else -1) and its
 * code is returned; that handle's sphgpu_last_error has the message.
 * Replaces: running one Spheral problem per process for a parameter study
 * (no single reference entry point; the SpheralController loop,
 * src/SimulationControl/SpheralController.py, per box). */
int sphgpu_ensemble_advance(sphgpu_handle* handles, int nboxes, int nsteps, double max_time, int nthreads,
                            int* failed);

/* Download / overwrite a field by reference name (caller node order).
 * Names: position velocity mass massDensity specificThermalEnergy H pressure
 * soundSpeed omegaGradh massDensitySum normalization DxDt DvDt DrhoDt DepsDt
 * DvDx internalDvDx gradRho M localM maxViscousPressure effViscousPressure
 * XSPHWeightSum XSPHDeltaV DHDt Hideal massZerothMoment massFirstMoment
 * DvDtGravity potential DepsDtCompatible numNeighbors
 * ArtificialViscosityVelocityGradient (limited Q) massSecondMoment (ASPH).
 * H, Hideal and DHDt are 6-component symmetric tensors.
 * *ncomp (may be NULL) receives the component count.
 * Replaces: State/StateDerivatives::fields(name, ...) (src/DataBase/State.hh:58-118). */
int sphgpu_get_field(sphgpu_handle h, const char* name, double* out, int* ncomp);
int sphgpu_set_field(sphgpu_handle h, const char* name, const double* in);

/* Overwrite the evolved state of all nodes from host arrays in caller order
 * (any pointer may be NULL to keep that field).  The package's derivative
 * fields stay on the device, as SPHBase owns its derivative FieldLists
 * (src/SPH/SPHBase.hh:223-253) while the NodeLists own the state.
 * Arrays in page-locked (pinned) host memory are read in place by the
 * device over the host link, in stream order: keep them unchanged until the
 * next call that synchronises (step, download_state, synchronize).  Pageable
 * arrays are copied through a device staging buffer.
 * Replaces: the State field references handed to Physics::evaluateDerivatives
 * (src/Physics/Physics.hh:49-60) when the host owns the FieldLists. */
int sphgpu_upload_state(sphgpu_handle h, const double* pos, const double* vel, const double* mass, const double* rho,
                        const double* eps, const double* H);

/* Copy the evolved state back to host arrays in caller order (NULL skips a
 * field); pinned arrays are written in place by the device.  Returns when
 * the arrays hold the state.
 * Replaces: reading the NodeList FieldLists after Integrator::step. */
int sphgpu_download_state(sphgpu_handle h, double* pos, double* vel, double* rho, double* eps, double* H);

/* Ordered neighbour pairs (i, j, image) in caller node indices; image packs
 * 2 bits per axis (0 none, 1 low-side image / lo mirror, 2 high-side image /
 * hi mirror).  Call with i == NULL to get *npairs only.
 * Replaces: ConnectivityMap::nodePairList (src/Neighbor/ConnectivityMap.hh). */
int sphgpu_get_pairs(sphgpu_handle h, int* i, int* j, int* image, long* npairs);

/* Conserved totals in FP64: {mass, px, py, pz, kinetic, thermal, gravity
 * potential (1/2 sum m phi), total}.  Replaces: SpheralConservation
 * (src/SimulationControl/SpheralConservation.py:54-150). */
int sphgpu_conservation(sphgpu_handle h, double out[8]);

/* Integrator clock: time, last dt, cycle. */
int sphgpu_get_time(sphgpu_handle h, double* time, double* last_dt, long* cycle);
int sphgpu_num_particles(sphgpu_handle h, long* n);

/* Per-kernel device timing.  enable != 0 records CUDA events around each
 * kernel of the next calls; sphgpu_profile_get returns, for kernel `name`,
 * the number of launches and the summed milliseconds. */
int sphgpu_profile_enable(sphgpu_handle h, int enable);
int sphgpu_profile_get(sphgpu_handle h, const char* name, long* launches, double* ms);
int sphgpu_profile_reset(sphgpu_handle h);
/* Number of kernels this library launched on the handle since creation. */
int sphgpu_launch_count(sphgpu_handle h, long* launches);
/* Device timing of everything issued on the handle's stream between the two
 * calls (CUDA events on that stream); stop waits for the stop event. */
int sphgpu_timer_start(sphgpu_handle h);
int sphgpu_timer_stop(sphgpu_handle h, double* ms);
/* Ordered neighbour entries of the current lists (2x the unordered pairs). */
int sphgpu_neighbor_count(sphgpu_handle h, long* entries);
/* Mixed-mode pair kernel variant (register budget and loop form: software
 * pipelined, or two / four neighbour slots per iteration; the count depends
 * on the configured hydro and smoothing scale).  By default (-1) the fastest
 * is picked by timing each at the first evaluation for a problem size and
 * again two evaluations later; sphgpu_set_pair_variant pins one
 * (0 .. *nvariants-1 from sphgpu_get_pair_variant), or -1 to re-enable the
 * autotuner.  Every variant gives the same bits.  sphgpu_get_pair_variant
 * returns the variant in use (-1 before the first mixed-mode evaluation).
 * No reference counterpart (tuning only). */
int sphgpu_set_pair_variant(sphgpu_handle h, int variant);
int sphgpu_get_pair_variant(sphgpu_handle h, int* variant, int* nvariants);
/* Lanes per work group of the neighbour search (8, 16 or 32), picked by
 * timing each width once per problem size; sphgpu_set_neighbor_width pins
 * one (taking effect at the next list build), or 0 to re-enable the
 * autotuner.  The lists, entry order included, are the same for every
 * width.  No reference counterpart (tuning only). */
int sphgpu_set_neighbor_width(sphgpu_handle h, int width);
int sphgpu_get_neighbor_width(sphgpu_handle h, int* width);
/* Batch depth of the mixed-mode compatible-energy sweep (slots whose loads
 * are issued together), autotuned like the pair variant; -1 re-enables the
 * autotuner.  Every depth sums in slot order, so the energies are the same
 * for every variant.  No reference counterpart (tuning only). */
int sphgpu_set_energy_variant(sphgpu_handle h, int variant);
int sphgpu_get_energy_variant(sphgpu_handle h, int* variant, int* nvariants);

/* Checkpoint and restart.  Replaces: SPHBase::dumpState / restoreState
 * (src/SPH/SPHBase.cc:711-768) with the integrator's time, last dt and cycle,
 * written through the caller's FileIO.  sphgpu_checkpoint_size gives the byte
 * count of the image of the current state; sphgpu_checkpoint copies it into
 * the caller's buffer; sphgpu_restore loads an image into a handle created
 * with the same configuration, NodeLists and boundaries (no set_particles
 * needed).  The image keeps the library's internal node order and kernel
 * variant, so a restored run continues bitwise as the uninterrupted one.
 * SPHGPU_E_ARG for a buffer that is not such an image (wrong tag or version,
 * short, a node order that is not a permutation, NodeList ids out of range),
 * SPHGPU_E_STATE for an image of another precision mode, viscosity, smoothing
 * scale, hydro package, RK volume type, kernel table or NodeList set. */
int sphgpu_checkpoint_size(sphgpu_handle h, size_t* bytes);
int sphgpu_checkpoint(sphgpu_handle h, void* buffer, size_t bytes);
int sphgpu_restore(sphgpu_handle h, const void* buffer, size_t bytes);

/* Wait for all work on the handle's stream. */
int sphgpu_synchronize(sphgpu_handle h);

/* Allocation-free conserved totals.  This entry point has no counterpart in
 * the reference; it exists for callers that cannot allocate GPU memory while
 * they run -- codes that hand the library slices of their own pre-allocated
 * device pools, code inside regions where an allocation would synchronise the
 * device, drivers whose footprint must stay fixed once started.  It computes
 * the same {mass, px, py, pz, kinetic, thermal, 1/2 sum m phi, total} as
 * sphgpu_conservation from caller device arrays (mass[n], vel[3n] in Vector
 * layout, eps[n], pot[n] or NULL) into the caller device array out[8], and
 * calls no cudaMalloc, cudaFree or allocating library routine.  Its scratch is
 * a fixed 57,344-byte array inside the library that every GPU loading the
 * library holds until the process exits and that all calls on a device share:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * The first call on a device looks up the scratch address (make it before any
 * stream capture).  n must be 1..67,108,864 (SPHGPU_E_OVERFLOW above that,
 * SPHGPU_E_ARG for n <= 0 or null pointers).  Work is queued on `stream` (a
 * cudaStream_t, NULL for the default stream) and is not waited for. */
int sphgpu_conservation_noalloc(const double* mass, const double* vel, const double* eps, const double* pot, long n,
                                double* out, void* stream);

/* Domain decomposition (the halo exchange of a single run spread over
 * several handles, one per domain, each on its own GPU or sharing one).
 * A domain's handle holds its owned nodes first (caller indices
 * 0..n-n_ghost-1) and then n_ghost halo copies of other domains' nodes that
 * lie within a kernel support of it; the caller builds that node set (for
 * instance from sphgpu_checkpoint images, whose rows sphgpu_image_layout
 * describes) and registers it with sphgpu_set_domain.  Halo copies are read
 * as neighbours by every sweep, take no part in the time-step vote, and are
 * refreshed during sphgpu_step through `fn`, called once per step at each of
 * these points, in this order, on every domain:
 *   SPHGPU_EXCHANGE_DENSITY  after the start-of-step density sum: mass density
 *   SPHGPU_EXCHANGE_DT       *dt holds this domain's vote; fn stores the
 *                            smallest vote of all domains there
 *   SPHGPU_EXCHANGE_OMEGA    after the mid-step grad-h correction (when on)
 *   SPHGPU_EXCHANGE_DERIVS   after the mid-step derivatives: DvDt (3), DepsDt
 * At a row point fn gathers, with sphgpu_exchange_get, the rows of the owned
 * nodes other domains hold as halo copies, sends them, and stores the rows
 * of its own halo (in halo caller order) with sphgpu_exchange_put.  fn
 * returns 0, or non-zero to fail the step with SPHGPU_E_STATE.  Everything
 * else a halo copy needs during the step it computes itself, bitwise as its
 * owner does, from the rows it started the step with.  n_ghost = 0 and
 * fn = NULL end the decomposition.  Gravity and CRKSPH are not covered
 * (SPHGPU_E_UNSUPPORTED).
 * Replaces: DistributedBoundary (src/Distributed/DistributedBoundary.cc:
 * setControlAndGhostNodes, applyGhostBoundaries, finalizeGhostBoundary) and
 * the global time-step minimum of Integrator::selectDt
 * (src/Integrator/Integrator.cc:152-153). */
#define SPHGPU_EXCHANGE_DENSITY 1
#define SPHGPU_EXCHANGE_DT 2
#define SPHGPU_EXCHANGE_OMEGA 3
#define SPHGPU_EXCHANGE_DERIVS 4
typedef int (*sphgpu_exchange_fn)(void* user, int point, double* dt);
int sphgpu_set_domain(sphgpu_handle h, long n_ghost, sphgpu_exchange_fn fn, void* user);
/* Values per node exchanged at `point` (0 for SPHGPU_EXCHANGE_DT). */
int sphgpu_exchange_width(sphgpu_handle h, int point, int* width);
/* Rows (width values each) of the owned nodes idx[0..count) into out. */
int sphgpu_exchange_get(sphgpu_handle h, int point, const int* idx, long count, double* out);
/* Rows of the n_ghost halo copies, in halo caller order, from in. */
int sphgpu_exchange_put(sphgpu_handle h, int point, const double* in);
/* Layout of a checkpoint image: header bytes, then nrows rows of n doubles
 * (one per carried field, internal node order), then n ints of caller index
 * and n ints of NodeList id.  *row (if field is not NULL) is the first row of
 * the named field (e.g. "position": rows row..row+2 hold x, y, z). */
int sphgpu_image_layout(sphgpu_handle h, const char* field, size_t* header_bytes, int* row, int* nrows);

#ifdef __cplusplus
}
#endif
#endif /* SPHGPU_H */
