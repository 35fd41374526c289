// Minimal stand-ins for the Spheral types that include/sphgpu_spheral.hh
// uses, so the GpuSPH package compiles and runs in this repository's tests
// without Spheral's build (its TPLs are not available here).  Names and
// signatures follow the reference headers (src/Geometry/Dimension.hh,
// src/Field/FieldList.hh, src/DataBase/{DataBase,State,StateDerivatives}.hh,
// src/Physics/Physics.hh, src/Hydro/HydroFieldNames.hh); only the members
// the package calls exist.  Test infrastructure only.
#ifndef SPHERAL_STUB_HH
#define SPHERAL_STUB_HH

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace Spheral {

struct GeomVector3 {
  double v[3] = {0.0, 0.0, 0.0};
  GeomVector3() = default;
  GeomVector3(double x, double y, double z) : v{x, y, z} {}
  double operator()(int a) const { return v[a]; }
  double& operator()(int a) { return v[a]; }
  static GeomVector3 zero() { return GeomVector3(); }
};

struct GeomTensor3 {
  double m[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  GeomTensor3() = default;
  GeomTensor3(double a, double b, double c, double d, double e, double f, double g, double h, double i)
      : m{a, b, c, d, e, f, g, h, i} {}
  double operator()(int r, int c) const { return m[3 * r + c]; }
  static GeomTensor3 zero() { return GeomTensor3(); }
};

// Symmetric tensor: the six upper-triangle elements (the 9-argument
// constructor keeps the upper triangle, as GeomSymmetricTensor does).
struct GeomSymmetricTensor3 {
  double m[6] = {0, 0, 0, 0, 0, 0};
  GeomSymmetricTensor3() = default;
  GeomSymmetricTensor3(double xx, double xy, double xz, double, double yy, double yz, double, double, double zz)
      : m{xx, xy, xz, yy, yz, zz} {}
  double operator()(int r, int c) const {
    if (r > c) std::swap(r, c);
    static const int idx[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    return m[idx[r][c]];
  }
  static GeomSymmetricTensor3 zero() { return GeomSymmetricTensor3(); }
};

template <int nDimValue>
struct Dim {
  static constexpr int nDim = nDimValue;
  using Scalar = double;
  using Vector = GeomVector3;
  using Tensor = GeomTensor3;
  using SymTensor = GeomSymmetricTensor3;
};

template <typename Dimension, typename DataType>
class Field {
 public:
  Field(std::string name, size_t n, DataType value) : mName(std::move(name)), mData(n, value) {}
  unsigned numInternalElements() const { return (unsigned)mData.size(); }
  DataType& operator()(unsigned i) { return mData.at(i); }
  const DataType& operator()(unsigned i) const { return mData.at(i); }
  const std::string& name() const { return mName; }

 private:
  std::string mName;
  std::vector<DataType> mData;
};

// A list of shared fields, one per NodeList (copies share the fields).
template <typename Dimension, typename DataType>
class FieldList {
 public:
  unsigned numFields() const { return (unsigned)mFields.size(); }
  Field<Dimension, DataType>* operator[](unsigned k) const { return mFields.at(k).get(); }
  void append(std::shared_ptr<Field<Dimension, DataType>> f) { mFields.push_back(std::move(f)); }

 private:
  std::vector<std::shared_ptr<Field<Dimension, DataType>>> mFields;
};

template <typename Dimension>
class DataBase {
 public:
  using Scalar = typename Dimension::Scalar;
  using Vector = typename Dimension::Vector;
  using SymTensor = typename Dimension::SymTensor;
  // One fluid NodeList of n nodes per entry of sizes.
  explicit DataBase(const std::vector<size_t>& sizes) : mSizes(sizes) {
    mPosition = newFluidFieldList(Vector::zero(), "position");
    mVelocity = newFluidFieldList(Vector::zero(), "velocity");
    mMass = newFluidFieldList(0.0, "mass");
    mRho = newFluidFieldList(0.0, "mass density");
    mEps = newFluidFieldList(0.0, "specific thermal energy");
    mH = newFluidFieldList(SymTensor::zero(), "H");
  }
  unsigned numFluidNodeLists() const { return (unsigned)mSizes.size(); }
  FieldList<Dimension, Vector> fluidPosition() const { return mPosition; }
  FieldList<Dimension, Vector> fluidVelocity() const { return mVelocity; }
  FieldList<Dimension, Scalar> fluidMass() const { return mMass; }
  FieldList<Dimension, Scalar> fluidMassDensity() const { return mRho; }
  FieldList<Dimension, Scalar> fluidSpecificThermalEnergy() const { return mEps; }
  FieldList<Dimension, SymTensor> fluidHfield() const { return mH; }
  template <typename T>
  FieldList<Dimension, T> newFluidFieldList(const T value, const std::string& name) const {
    FieldList<Dimension, T> fl;
    for (size_t n : mSizes) fl.append(std::make_shared<Field<Dimension, T>>(name, n, value));
    return fl;
  }

 private:
  std::vector<size_t> mSizes;
  FieldList<Dimension, Vector> mPosition, mVelocity;
  FieldList<Dimension, Scalar> mMass, mRho, mEps;
  FieldList<Dimension, SymTensor> mH;
};

// Field storage keyed by field name (State and StateDerivatives).
template <typename Dimension>
class FieldStore {
 public:
  using Scalar = typename Dimension::Scalar;
  using Vector = typename Dimension::Vector;
  using Tensor = typename Dimension::Tensor;
  using SymTensor = typename Dimension::SymTensor;
  void enroll(const FieldList<Dimension, Scalar>& fl) { mS[fl[0]->name()] = fl; }
  void enroll(const FieldList<Dimension, Vector>& fl) { mV[fl[0]->name()] = fl; }
  void enroll(const FieldList<Dimension, Tensor>& fl) { mT[fl[0]->name()] = fl; }
  void enroll(const FieldList<Dimension, SymTensor>& fl) { mY[fl[0]->name()] = fl; }
  FieldList<Dimension, Scalar> fields(const std::string& k, const Scalar&) const { return find(mS, k); }
  FieldList<Dimension, Vector> fields(const std::string& k, const Vector&) const { return find(mV, k); }
  FieldList<Dimension, Tensor> fields(const std::string& k, const Tensor&) const { return find(mT, k); }
  FieldList<Dimension, SymTensor> fields(const std::string& k, const SymTensor&) const { return find(mY, k); }

 private:
  template <typename M>
  static typename M::mapped_type find(const M& m, const std::string& k) {
    auto it = m.find(k);
    if (it == m.end()) throw std::runtime_error("no field registered as '" + k + "'");
    return it->second;
  }
  std::map<std::string, FieldList<Dimension, Scalar>> mS;
  std::map<std::string, FieldList<Dimension, Vector>> mV;
  std::map<std::string, FieldList<Dimension, Tensor>> mT;
  std::map<std::string, FieldList<Dimension, SymTensor>> mY;
};
template <typename Dimension> class State : public FieldStore<Dimension> {};
template <typename Dimension> class StateDerivatives : public FieldStore<Dimension> {};

template <typename Dimension>
class Physics {
 public:
  using Scalar = typename Dimension::Scalar;
  using TimeStepType = std::pair<double, std::string>;
  virtual ~Physics() = default;
  virtual void evaluateDerivatives(const Scalar time, const Scalar dt, const DataBase<Dimension>& dataBase,
                                   const State<Dimension>& state, StateDerivatives<Dimension>& derivs) const = 0;
  virtual TimeStepType dt(const DataBase<Dimension>& dataBase, const State<Dimension>& state,
                          const StateDerivatives<Dimension>& derivs, const Scalar currentTime) const = 0;
  virtual void registerState(DataBase<Dimension>& dataBase, State<Dimension>& state) = 0;
  virtual void registerDerivatives(DataBase<Dimension>& dataBase, StateDerivatives<Dimension>& derivs) = 0;
  virtual std::string label() const = 0;
  virtual void initializeProblemStartupDependencies(DataBase<Dimension>&, State<Dimension>&,
                                                    StateDerivatives<Dimension>&) {}
  virtual void finalize(const Scalar, const Scalar, DataBase<Dimension>&, State<Dimension>&,
                        StateDerivatives<Dimension>&) {}
  virtual bool requireConnectivity() const { return true; }
  virtual Scalar extraEnergy() const { return 0.0; }
};

struct HydroFieldNames {
  static inline const std::string mass = "mass";
  static inline const std::string position = "position";
  static inline const std::string velocity = "velocity";
  static inline const std::string H = "H";
  static inline const std::string velocityGradient = "velocity gradient";
  static inline const std::string internalVelocityGradient = "internal velocity gradient";
  static inline const std::string hydroAcceleration = "delta velocity hydro";
  static inline const std::string massDensity = "mass density";
  static inline const std::string normalization = "normalization";
  static inline const std::string specificThermalEnergy = "specific thermal energy";
  static inline const std::string maxViscousPressure = "max viscous pressure";
  static inline const std::string effectiveViscousPressure = "effective viscous pressure";
  static inline const std::string XSPHDeltaV = "XSPH delta vi";
  static inline const std::string XSPHWeightSum = "XSPH weight sum";
  static inline const std::string pressure = "pressure";
  static inline const std::string soundSpeed = "sound speed";
  static inline const std::string omegaGradh = "grad h corrections";
  static inline const std::string M_SPHCorrection = "M SPH gradient correction";
  static inline const std::string massDensityGradient = "mass density gradient";
};

}  // namespace Spheral

#endif
