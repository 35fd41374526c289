// Drives the GpuSPH Physics package (include/sphgpu_spheral.hh) the way a
// Spheral integrator does, compiled with g++ against include/sphgpu.h and
// linked with libsphgpu.so:
//   registerState -> registerDerivatives -> initializeProblemStartupDependencies
//   -> evaluateDerivatives -> dt -> stepOnDevice x nsteps
// Input and output are flat float64 files written / read by
// tests/test_gpu_cpp_shim.py, which compares the results with the oracle.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <vector>

#include "sphgpu_spheral.hh"

using namespace Spheral;
using D = Dim<3>;

namespace {
std::vector<double> readAll(const char* path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error(std::string("cannot open ") + path);
  f.seekg(0, std::ios::end);
  const size_t bytes = (size_t)f.tellg();
  f.seekg(0);
  std::vector<double> v(bytes / sizeof(double));
  f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)bytes);
  return v;
}
template <typename T> void dump(std::ofstream& o, const FieldList<D, T>& fl, int nc) {
  for (unsigned k = 0; k < fl.numFields(); ++k)
    for (unsigned i = 0; i < fl[k]->numInternalElements(); ++i)
      o.write(reinterpret_cast<const char*>(&(*fl[k])(i)), nc * sizeof(double));
}
}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    std::cerr << "usage: physics_shim problem.bin out_prefix\n";
    return 2;
  }
  try {
    const std::vector<double> in = readAll(argv[1]);
    size_t q = 0;
    auto next = [&]() { return in.at(q++); };
    const long n = (long)next();
    const int nsteps = (int)next();
    const int nbcs = (int)next();
    sphgpu_config cfg;
    sphgpu_default_config(&cfg);
    cfg.cfl = next();
    cfg.compatible_energy = (int)next();
    cfg.gradh_correction = (int)next();
    cfg.xsph = (int)next();
    cfg.correct_velocity_gradient = (int)next();
    cfg.Cl = next();
    cfg.Cq = next();
    cfg.dt_min = next();
    cfg.dt_max = next();
    cfg.dt_growth = next();
    cfg.last_dt = next();
    cfg.precision = (int)next();
    cfg.viscosity = (int)next();
    GpuNodeListParams nl;
    nl.nPerh = next(); nl.hmin = next(); nl.hmax = next(); nl.rhoMin = next(); nl.rhoMax = next(); nl.gamma = next();
    std::vector<GpuPlanarBoundary> bcs;
    for (int b = 0; b < nbcs; ++b) {
      GpuPlanarBoundary g;
      g.type = (int)next(); g.axis = (int)next(); g.lo = next(); g.hi = next(); g.wallHigh = (int)next();
      bcs.push_back(g);
    }
    // One fluid NodeList holding the problem's nodes.
    DataBase<D> db({(size_t)n});
    {
      auto pos = db.fluidPosition();
      auto vel = db.fluidVelocity();
      auto m = db.fluidMass();
      auto rho = db.fluidMassDensity();
      auto eps = db.fluidSpecificThermalEnergy();
      auto H = db.fluidHfield();
      const size_t p0 = q, v0 = p0 + 3 * n, m0 = v0 + 3 * n, r0 = m0 + n, e0 = r0 + n, h0 = e0 + n;
      for (long i = 0; i < n; ++i) {
        (*pos[0])(i) = D::Vector(in.at(p0 + 3 * i), in.at(p0 + 3 * i + 1), in.at(p0 + 3 * i + 2));
        (*vel[0])(i) = D::Vector(in.at(v0 + 3 * i), in.at(v0 + 3 * i + 1), in.at(v0 + 3 * i + 2));
        (*m[0])(i) = in.at(m0 + i);
        (*rho[0])(i) = in.at(r0 + i);
        (*eps[0])(i) = in.at(e0 + i);
        const double* h = &in.at(h0 + 6 * i);
        (*H[0])(i) = D::SymTensor(h[0], h[1], h[2], h[1], h[3], h[4], h[2], h[4], h[5]);
      }
    }
    GpuSPH<D> pkg(cfg, {nl}, bcs);
    Physics<D>& physics = pkg;   // everything below goes through the Physics interface
    State<D> state;
    StateDerivatives<D> derivs;
    physics.registerState(db, state);
    physics.registerDerivatives(db, derivs);
    physics.initializeProblemStartupDependencies(db, state, derivs);
    physics.evaluateDerivatives(0.0, cfg.last_dt, db, state, derivs);
    const auto vote = physics.dt(db, state, derivs, 0.0);
    {
      std::ofstream o(std::string(argv[2]) + "_derivs.bin", std::ios::binary);
      dump(o, derivs.fields(HydroFieldNames::hydroAcceleration, D::Vector::zero()), 3);
      dump(o, derivs.fields("delta " + HydroFieldNames::specificThermalEnergy, 0.0), 1);
      dump(o, derivs.fields(HydroFieldNames::velocityGradient, D::Tensor::zero()), 9);
      dump(o, derivs.fields("new " + HydroFieldNames::massDensity, 0.0), 1);
      dump(o, derivs.fields("new " + HydroFieldNames::H, D::SymTensor::zero()), 6);
      dump(o, derivs.fields("delta " + HydroFieldNames::H, D::SymTensor::zero()), 6);
      dump(o, derivs.fields(HydroFieldNames::maxViscousPressure, 0.0), 1);
      dump(o, state.fields(HydroFieldNames::pressure, 0.0), 1);
      o.write(reinterpret_cast<const char*>(&vote.first), sizeof(double));
    }
    std::cout << "label " << physics.label() << " dt " << vote.first << " (" << vote.second << ")\n";
    double t = 0.0;
    for (int k = 0; k < nsteps; ++k) {
      bool accepted = false;
      t += pkg.stepOnDevice(state, 1.0e300, accepted);
      if (!accepted) throw std::runtime_error("step rejected");
    }
    double time = 0.0, lastDt = 0.0;
    long cycle = 0;
    pkg.deviceClock(time, lastDt, cycle);
    physics.finalize(time, lastDt, db, state, derivs);
    {
      std::ofstream o(std::string(argv[2]) + "_state.bin", std::ios::binary);
      o.write(reinterpret_cast<const char*>(&time), sizeof(double));
      dump(o, state.fields(HydroFieldNames::position, D::Vector::zero()), 3);
      dump(o, state.fields(HydroFieldNames::velocity, D::Vector::zero()), 3);
      dump(o, state.fields(HydroFieldNames::massDensity, 0.0), 1);
      dump(o, state.fields(HydroFieldNames::specificThermalEnergy, 0.0), 1);
      dump(o, state.fields(HydroFieldNames::H, D::SymTensor::zero()), 6);
      dump(o, state.fields(HydroFieldNames::pressure, 0.0), 1);
    }
    std::cout << "steps " << cycle << " time " << time << " sum of dt " << t << "\n";
  } catch (const std::exception& e) {
    std::cerr << "physics_shim: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
