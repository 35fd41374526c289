// GpuSPH<Dimension>: a Spheral Physics package backed by libsphgpu, the
// sm_103a SPH hydro step behind include/sphgpu.h.
//
// Drop-in for the package SPH(...) builds (src/SPH/SPHHydros.py:9-156,
// SPH<Dim<3>> in src/SPH/SPH.cc) on the ideal-gas path.  It implements the
// Physics<Dimension> interface of src/Physics/Physics.hh:49-193:
//
//   registerState          SPHBase::registerState (src/SPH/SPHBase.cc:203-263): the NodeList
//                          state FieldLists plus the package's pressure, sound speed and
//                          grad-h correction
//   registerDerivatives    SPHBase::registerDerivatives (SPHBase.cc:271-320) and
//                          SmoothingScaleBase::registerDerivatives: the derivative
//                          FieldLists under the reference's keys ("delta position",
//                          "delta velocity hydro", "new H", ...)
//   initializeProblemStartupDependencies
//                          SPHBase.cc:152-197: uploads the nodes (sphgpu_set_particles) and
//                          computes P, c and Omega on the GPU (sphgpu_initialize)
//   evaluateDerivatives    SPH::evaluateDerivatives (SPH.cc:143-555) + SPHSmoothingScale: the
//                          state is uploaded (sphgpu_upload_state), evaluated
//                          (sphgpu_evaluate_derivatives) and every registered derivative
//                          FieldList is filled from the device (sphgpu_get_field)
//   dt                     GenericHydro::dt (src/Physics/GenericHydro.cc:113-381) -> sphgpu_dt
//   finalize               SPHBase::finalize: pressure, sound speed and Omega of the final
//                          state read back into the package's FieldLists
//   label, requireConnectivity, extraEnergy
//
// plus the device-resident fast path stepOnDevice(): one whole
// CheapSynchronousRK2 step (src/Integrator/CheapSynchronousRK2.cc:40-132) on
// the GPU (sphgpu_step) with the state copied in and out, for an integrator
// that hands the step to the package.
//
// Errors: every non-zero status becomes a std::runtime_error carrying
// sphgpu_last_error (Spheral's VERIFY2 throws the same way, src/Utilities/DBC.hh);
// no exception crosses the C ABI.  Field flattening follows DataBase order:
// NodeList k's internal nodes follow those of NodeLists 0..k-1, and the
// NodeList id of a node is k.
//
// The header needs Spheral's own headers on the include path (it is meant to
// live in src/GPU/); it uses only: Dimension::{Scalar, Vector, Tensor,
// SymTensor, nDim}; FieldList::numFields / operator[] and Field::
// numInternalElements / operator(); DataBase::fluid* accessors,
// numFluidNodeLists and newFluidFieldList; State/StateDerivatives::enroll and
// fields(key, dummy); HydroFieldNames.
#ifndef SPHGPU_SPHERAL_HH
#define SPHGPU_SPHERAL_HH

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "DataBase/DataBase.hh"
#include "DataBase/State.hh"
#include "DataBase/StateDerivatives.hh"
#include "Field/FieldList.hh"
#include "Hydro/HydroFieldNames.hh"
#include "Physics/Physics.hh"
#include "sphgpu.h"

namespace Spheral {

// Per-NodeList parameters the package needs (FluidNodeList + GammaLawGas).
struct GpuNodeListParams {
  double nPerh, hmin, hmax, rhoMin, rhoMax, gamma;
};

// An axis-aligned PeriodicBoundary (type SPHGPU_BOUNDARY_PERIODIC, planes at
// lo and hi) or ReflectingBoundary (type SPHGPU_BOUNDARY_REFLECTING, one wall).
struct GpuPlanarBoundary {
  int type, axis;
  double lo, hi;
  int wallHigh;
};

template <typename Dimension>
class GpuSPH : public Physics<Dimension> {
  static_assert(Dimension::nDim == 3, "the GPU SPH step is three-dimensional");

 public:
  using Scalar = typename Dimension::Scalar;
  using Vector = typename Dimension::Vector;
  using Tensor = typename Dimension::Tensor;
  using SymTensor = typename Dimension::SymTensor;
  using TimeStepType = typename Physics<Dimension>::TimeStepType;

  GpuSPH(const sphgpu_config& cfg, const std::vector<GpuNodeListParams>& lists,
         const std::vector<GpuPlanarBoundary>& boundaries)
      : mCfg(cfg) {
    check(sphgpu_create(&cfg, &mH), "sphgpu_create");
    for (size_t k = 0; k < lists.size(); ++k) {
      const GpuNodeListParams& p = lists[k];
      check(sphgpu_set_nodelist(mH, (int)k, p.nPerh, p.hmin, p.hmax, p.rhoMin, p.rhoMax, p.gamma),
            "sphgpu_set_nodelist");
    }
    for (const GpuPlanarBoundary& b : boundaries)
      check(sphgpu_add_boundary(mH, b.type, b.axis, b.lo, b.hi, b.wallHigh), "sphgpu_add_boundary");
  }
  GpuSPH(const GpuSPH&) = delete;
  GpuSPH& operator=(const GpuSPH&) = delete;
  virtual ~GpuSPH() {
    if (mH) sphgpu_destroy(mH);
  }

  //--------------------------------------------------------------------------
  // Physics interface
  //--------------------------------------------------------------------------
  virtual void registerState(DataBase<Dimension>& dataBase, State<Dimension>& state) override {
    mPosition = dataBase.fluidPosition();
    mVelocity = dataBase.fluidVelocity();
    mMass = dataBase.fluidMass();
    mMassDensity = dataBase.fluidMassDensity();
    mSpecificThermalEnergy = dataBase.fluidSpecificThermalEnergy();
    mHfield = dataBase.fluidHfield();
    if (mPressure.numFields() == 0) {
      mPressure = dataBase.newFluidFieldList(0.0, HydroFieldNames::pressure);
      mSoundSpeed = dataBase.newFluidFieldList(0.0, HydroFieldNames::soundSpeed);
      mOmegaGradh = dataBase.newFluidFieldList(1.0, HydroFieldNames::omegaGradh);
    }
    state.enroll(mPosition);
    state.enroll(mVelocity);
    state.enroll(mMass);
    state.enroll(mMassDensity);
    state.enroll(mSpecificThermalEnergy);
    state.enroll(mHfield);
    state.enroll(mPressure);
    state.enroll(mSoundSpeed);
    state.enroll(mOmegaGradh);
  }

  virtual void registerDerivatives(DataBase<Dimension>& dataBase, StateDerivatives<Dimension>& derivs) override {
    if (mDvDt.numFields() == 0) {
      mDxDt = dataBase.newFluidFieldList(Vector::zero(), "delta " + HydroFieldNames::position);
      mDvDt = dataBase.newFluidFieldList(Vector::zero(), HydroFieldNames::hydroAcceleration);
      mDrhoDt = dataBase.newFluidFieldList(0.0, "delta " + HydroFieldNames::massDensity);
      mDepsDt = dataBase.newFluidFieldList(0.0, "delta " + HydroFieldNames::specificThermalEnergy);
      mDvDx = dataBase.newFluidFieldList(Tensor::zero(), HydroFieldNames::velocityGradient);
      mInternalDvDx = dataBase.newFluidFieldList(Tensor::zero(), HydroFieldNames::internalVelocityGradient);
      mGradRho = dataBase.newFluidFieldList(Vector::zero(), HydroFieldNames::massDensityGradient);
      mM = dataBase.newFluidFieldList(Tensor::zero(), HydroFieldNames::M_SPHCorrection);
      mLocalM = dataBase.newFluidFieldList(Tensor::zero(), "local " + HydroFieldNames::M_SPHCorrection);
      mMassDensitySum = dataBase.newFluidFieldList(0.0, "new " + HydroFieldNames::massDensity);
      mNormalization = dataBase.newFluidFieldList(0.0, HydroFieldNames::normalization);
      mXSPHWeightSum = dataBase.newFluidFieldList(0.0, HydroFieldNames::XSPHWeightSum);
      mXSPHDeltaV = dataBase.newFluidFieldList(Vector::zero(), HydroFieldNames::XSPHDeltaV);
      mMaxViscousPressure = dataBase.newFluidFieldList(0.0, HydroFieldNames::maxViscousPressure);
      mEffViscousPressure = dataBase.newFluidFieldList(0.0, HydroFieldNames::effectiveViscousPressure);
      mDHDt = dataBase.newFluidFieldList(SymTensor::zero(), "delta " + HydroFieldNames::H);
      mHideal = dataBase.newFluidFieldList(SymTensor::zero(), "new " + HydroFieldNames::H);
    }
    derivs.enroll(mDxDt);
    derivs.enroll(mDvDt);
    derivs.enroll(mDrhoDt);
    derivs.enroll(mDepsDt);
    derivs.enroll(mDvDx);
    derivs.enroll(mInternalDvDx);
    derivs.enroll(mGradRho);
    derivs.enroll(mM);
    derivs.enroll(mLocalM);
    derivs.enroll(mMassDensitySum);
    derivs.enroll(mNormalization);
    derivs.enroll(mXSPHWeightSum);
    derivs.enroll(mXSPHDeltaV);
    derivs.enroll(mMaxViscousPressure);
    derivs.enroll(mEffViscousPressure);
    derivs.enroll(mDHDt);
    derivs.enroll(mHideal);
  }

  virtual void initializeProblemStartupDependencies(DataBase<Dimension>& dataBase, State<Dimension>& state,
                                                    StateDerivatives<Dimension>& derivs) override {
    (void)dataBase;
    (void)derivs;
    gatherState(state);
    check(sphgpu_set_particles(mH, mN, mPos.data(), mVel.data(), mMassBuf.data(), mRho.data(), mEps.data(),
                               mH6.data(), mList.data()),
          "sphgpu_set_particles");
    check(sphgpu_initialize(mH), "sphgpu_initialize");
    scatter("pressure", mPressure);
    scatter("soundSpeed", mSoundSpeed);
    scatter("omegaGradh", mOmegaGradh);
  }

  virtual void evaluateDerivatives(const Scalar time, const Scalar dt, const DataBase<Dimension>& dataBase,
                                   const State<Dimension>& state,
                                   StateDerivatives<Dimension>& derivs) const override {
    (void)time;
    (void)dt;
    (void)dataBase;
    upload(state);
    check(sphgpu_evaluate_derivatives(mH), "sphgpu_evaluate_derivatives");
    fill(derivs, "DxDt", "delta " + HydroFieldNames::position, Vector::zero());
    fill(derivs, "DvDt", HydroFieldNames::hydroAcceleration, Vector::zero());
    fill(derivs, "DrhoDt", "delta " + HydroFieldNames::massDensity, 0.0);
    fill(derivs, "DepsDt", "delta " + HydroFieldNames::specificThermalEnergy, 0.0);
    fill(derivs, "DvDx", HydroFieldNames::velocityGradient, Tensor::zero());
    fill(derivs, "internalDvDx", HydroFieldNames::internalVelocityGradient, Tensor::zero());
    fill(derivs, "gradRho", HydroFieldNames::massDensityGradient, Vector::zero());
    fill(derivs, "M", HydroFieldNames::M_SPHCorrection, Tensor::zero());
    fill(derivs, "localM", "local " + HydroFieldNames::M_SPHCorrection, Tensor::zero());
    fill(derivs, "massDensitySum", "new " + HydroFieldNames::massDensity, 0.0);
    fill(derivs, "normalization", HydroFieldNames::normalization, 0.0);
    fill(derivs, "XSPHWeightSum", HydroFieldNames::XSPHWeightSum, 0.0);
    fill(derivs, "XSPHDeltaV", HydroFieldNames::XSPHDeltaV, Vector::zero());
    fill(derivs, "maxViscousPressure", HydroFieldNames::maxViscousPressure, 0.0);
    fill(derivs, "effViscousPressure", HydroFieldNames::effectiveViscousPressure, 0.0);
    fill(derivs, "DHDt", "delta " + HydroFieldNames::H, SymTensor::zero());
    fill(derivs, "Hideal", "new " + HydroFieldNames::H, SymTensor::zero());
  }

  virtual TimeStepType dt(const DataBase<Dimension>& dataBase, const State<Dimension>& state,
                          const StateDerivatives<Dimension>& derivs, const Scalar currentTime) const override {
    (void)dataBase;
    (void)derivs;
    (void)currentTime;
    upload(state);
    double v = 0.0;
    int reason = 0;
    check(sphgpu_dt(mH, &v, &reason), "sphgpu_dt");
    static const char* const names[] = {"sound speed", "artificial viscosity", "velocity divergence",
                                        "acceleration", "velocity magnitude", "pairwise velocity difference",
                                        "gravity"};
    return TimeStepType(v, std::string("GpuSPH: ") + names[(reason >= 0 && reason < 7) ? reason : 0]);
  }

  virtual void finalize(const Scalar time, const Scalar dt, DataBase<Dimension>& dataBase, State<Dimension>& state,
                        StateDerivatives<Dimension>& derivs) override {
    (void)time;
    (void)dt;
    (void)dataBase;
    (void)derivs;
    upload(state);
    scatter("pressure", mPressure);
    scatter("soundSpeed", mSoundSpeed);
    scatter("omegaGradh", mOmegaGradh);
  }

  virtual std::string label() const override { return "GpuSPH"; }
  virtual bool requireConnectivity() const override { return false; }   // the package builds its own cell lists
  virtual Scalar extraEnergy() const override {
    double out[8];
    check(sphgpu_conservation(mH, out), "sphgpu_conservation");
    return out[6];   // 1/2 sum m phi when gravity is on, else 0
  }

  //--------------------------------------------------------------------------
  // Device-resident path: one CheapSynchronousRK2 step of the whole state on
  // the GPU, bounded by maxTime.  The state FieldLists are uploaded first and
  // hold the new state afterwards.  Returns the step taken; status
  // SPHGPU_E_NAN (a non-finite state) is reported as a failed step (false in
  // `accepted`), as Integrator::step reports a rejected step.
  //--------------------------------------------------------------------------
  double stepOnDevice(State<Dimension>& state, const double maxTime, bool& accepted) {
    upload(state);
    double dt = 0.0;
    const int rc = sphgpu_step(mH, maxTime, &dt);
    accepted = (rc == SPHGPU_OK);
    if (rc == SPHGPU_E_NAN) return dt;
    check(rc, "sphgpu_step");
    check(sphgpu_download_state(mH, mPos.data(), mVel.data(), mRho.data(), mEps.data(), mH6.data()),
          "sphgpu_download_state");
    auto pos = state.fields(HydroFieldNames::position, Vector::zero());
    auto vel = state.fields(HydroFieldNames::velocity, Vector::zero());
    auto rho = state.fields(HydroFieldNames::massDensity, 0.0);
    auto eps = state.fields(HydroFieldNames::specificThermalEnergy, 0.0);
    auto H = state.fields(HydroFieldNames::H, SymTensor::zero());
    scatterHost(mPos, pos);
    scatterHost(mVel, vel);
    scatterHost(mRho, rho);
    scatterHost(mEps, eps);
    scatterHost(mH6, H);
    return dt;
  }

  // The integrator clock kept on the device (time, last dt, cycle).
  void deviceClock(double& time, double& lastDt, long& cycle) const {
    check(sphgpu_get_time(mH, &time, &lastDt, &cycle), "sphgpu_get_time");
  }

  sphgpu_handle handle() const { return mH; }

 private:
  sphgpu_config mCfg;
  sphgpu_handle mH = nullptr;
  long mN = 0;
  mutable std::vector<double> mPos, mVel, mMassBuf, mRho, mEps, mH6;
  std::vector<int> mList;
  FieldList<Dimension, Vector> mPosition, mVelocity;
  FieldList<Dimension, Scalar> mMass, mMassDensity, mSpecificThermalEnergy;
  FieldList<Dimension, SymTensor> mHfield;
  FieldList<Dimension, Scalar> mPressure, mSoundSpeed, mOmegaGradh;
  FieldList<Dimension, Vector> mDxDt, mDvDt, mGradRho, mXSPHDeltaV;
  FieldList<Dimension, Scalar> mDrhoDt, mDepsDt, mMassDensitySum, mNormalization, mXSPHWeightSum;
  FieldList<Dimension, Scalar> mMaxViscousPressure, mEffViscousPressure;
  FieldList<Dimension, Tensor> mDvDx, mInternalDvDx, mM, mLocalM;
  FieldList<Dimension, SymTensor> mDHDt, mHideal;

  void check(const int rc, const char* what) const {
    if (rc != SPHGPU_OK)
      throw std::runtime_error(std::string("GpuSPH: ") + what + " failed (" + std::to_string(rc) +
                               "): " + (mH ? sphgpu_last_error(mH) : ""));
  }

  // Flatten a FieldList in DataBase order: ncomp doubles per node.
  static void put(const Scalar& v, double* o) { o[0] = v; }
  static void put(const Vector& v, double* o) {
    for (int a = 0; a < 3; ++a) o[a] = v(a);
  }
  static void put(const Tensor& t, double* o) {
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) o[3 * r + c] = t(r, c);
  }
  static void put(const SymTensor& t, double* o) {
    o[0] = t(0, 0); o[1] = t(0, 1); o[2] = t(0, 2); o[3] = t(1, 1); o[4] = t(1, 2); o[5] = t(2, 2);
  }
  static void get(const double* o, Scalar& v) { v = o[0]; }
  static void get(const double* o, Vector& v) { v = Vector(o[0], o[1], o[2]); }
  static void get(const double* o, Tensor& t) { t = Tensor(o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7], o[8]); }
  static void get(const double* o, SymTensor& t) {
    t = SymTensor(o[0], o[1], o[2], o[1], o[3], o[4], o[2], o[4], o[5]);
  }
  static constexpr int ncomp(const Scalar*) { return 1; }
  static constexpr int ncomp(const Vector*) { return 3; }
  static constexpr int ncomp(const SymTensor*) { return 6; }
  static constexpr int ncomp(const Tensor*) { return 9; }

  template <typename T>
  static void flatten(const FieldList<Dimension, T>& fl, std::vector<double>& out) {
    const int nc = ncomp((const T*)nullptr);
    size_t n = 0;
    for (unsigned k = 0; k < fl.numFields(); ++k) n += fl[k]->numInternalElements();
    out.resize(n * nc);
    size_t q = 0;
    for (unsigned k = 0; k < fl.numFields(); ++k) {
      const auto& f = *fl[k];
      for (unsigned i = 0; i < f.numInternalElements(); ++i, q += nc) put(f(i), &out[q]);
    }
  }
  // FieldLists are taken by reference: a package-owned list copies its
  // fields when copied, so a copy would be filled instead of the list.
  template <typename T>
  static void scatterHost(const std::vector<double>& in, FieldList<Dimension, T>& fl) {
    const int nc = ncomp((const T*)nullptr);
    size_t q = 0;
    for (unsigned k = 0; k < fl.numFields(); ++k) {
      auto& f = *fl[k];
      for (unsigned i = 0; i < f.numInternalElements(); ++i, q += nc) get(&in[q], f(i));
    }
  }
  // Fill a FieldList from the device field `name`.
  template <typename T>
  void scatter(const char* name, FieldList<Dimension, T>& fl) const {
    std::vector<double> buf((size_t)mN * ncomp((const T*)nullptr));
    int nc = 0;
    check(sphgpu_get_field(mH, name, buf.data(), &nc), name);
    if (nc != ncomp((const T*)nullptr)) throw std::runtime_error(std::string("GpuSPH: component count of ") + name);
    scatterHost(buf, fl);
  }

  // Fill the derivative FieldList registered under `key` from device field `name`.
  template <typename T>
  void fill(StateDerivatives<Dimension>& derivs, const char* name, const std::string& key, const T& dummy) const {
    auto fl = derivs.fields(key, dummy);   // a list of references to the registered fields
    scatter(name, fl);
  }

  // Host copies of the state in DataBase order, and the NodeList ids.
  void gatherState(const State<Dimension>& state) {
    flatten(state.fields(HydroFieldNames::position, Vector::zero()), mPos);
    flatten(state.fields(HydroFieldNames::velocity, Vector::zero()), mVel);
    flatten(state.fields(HydroFieldNames::mass, 0.0), mMassBuf);
    flatten(state.fields(HydroFieldNames::massDensity, 0.0), mRho);
    flatten(state.fields(HydroFieldNames::specificThermalEnergy, 0.0), mEps);
    const auto Hfl = state.fields(HydroFieldNames::H, SymTensor::zero());
    flatten(Hfl, mH6);
    mN = (long)mMassBuf.size();
    mList.clear();
    for (unsigned k = 0; k < Hfl.numFields(); ++k) mList.insert(mList.end(), Hfl[k]->numInternalElements(), (int)k);
  }

  // Push the caller's current state (the integrator may have changed it).
  void upload(const State<Dimension>& state) const {
    flatten(state.fields(HydroFieldNames::position, Vector::zero()), mPos);
    flatten(state.fields(HydroFieldNames::velocity, Vector::zero()), mVel);
    flatten(state.fields(HydroFieldNames::mass, 0.0), mMassBuf);
    flatten(state.fields(HydroFieldNames::massDensity, 0.0), mRho);
    flatten(state.fields(HydroFieldNames::specificThermalEnergy, 0.0), mEps);
    flatten(state.fields(HydroFieldNames::H, SymTensor::zero()), mH6);
    if ((long)mMassBuf.size() != mN) throw std::runtime_error("GpuSPH: the node count changed since start-up");
    check(sphgpu_upload_state(mH, mPos.data(), mVel.data(), mMassBuf.data(), mRho.data(), mEps.data(), mH6.data()),
          "sphgpu_upload_state");
  }
};

}  // namespace Spheral

#endif  // SPHGPU_SPHERAL_HH
