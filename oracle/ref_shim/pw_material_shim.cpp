// Python binding for the reference's per-point material updaters.
//
// TEST INFRASTRUCTURE ONLY.  The reference (GMES) exposes its C++ updaters
// (src/pw_*.hh) to Python through a SWIG module generated from
// src/pw_material.i.  SWIG is not installed here, so this file is a
// hand-written pybind11 binding over the UNMODIFIED reference headers: it
// reproduces the class names (<Model><Comp>Real / Cmplx), the parameter
// structs with settable fields, the set() helpers of src/pw_material.i:215-348,
// the numpy argument checks and the exception mapping of
// src/pw_material.i:23-51.  It is compiled from the reference tree by
// oracle/build_ref.py into oracle/_ref/ and is used only to generate golden
// vectors and to pin the oracle; nothing in the product links it.

#include <complex>
#include <stdexcept>
#include <string>
#include <vector>

#include <pybind11/complex.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include "pw_material.hh"
#include "pw_dummy.hh"
#include "pw_const.hh"
#include "pw_dielectric.hh"
#include "pw_upml.hh"
#include "pw_cpml.hh"
#include "pw_drude.hh"
#include "pw_lorentz.hh"
#include "pw_dcp.hh"

namespace py = pybind11;
using namespace gmes;

namespace {

// Several reference updaters declare update_all/attach in a private section
// of the derived class; the calls below go through the public virtual
// interface of PwMaterial<T> (src/pw_material.hh:61-83).
//
// numpy.i's INPLACE_ARRAY3 / IN_ARRAY3 contract: exact dtype, ndim 3,
// C-contiguous; the in-place target must be writeable.
template <typename T>
struct Field {
  T* data;
  int d1, d2, d3;
};

template <typename T>
Field<T> as_field(py::array& a, bool inplace) {
  if (!a.dtype().is(py::dtype::of<T>()))
    throw py::type_error("array of the wrong type");
  if (a.ndim() != 3)
    throw py::type_error("array must have 3 dimensions");
  if (!(a.flags() & py::array::c_style))
    throw py::type_error("array must be contiguous");
  if (inplace && !a.writeable())
    throw py::type_error("array must be writeable");
  return Field<T>{static_cast<T*>(a.mutable_data()), static_cast<int>(a.shape(0)),
                  static_cast<int>(a.shape(1)), static_cast<int>(a.shape(2))};
}

std::vector<int> as_index(py::handle idx) {
  std::vector<int> out;
  for (auto v : idx) out.push_back(py::cast<int>(v));
  return out;
}

template <typename T, typename Cls>
void def_updater_methods(Cls& cls) {
  using C = typename Cls::type;
  cls.def(py::init<>())
      // attach/merge return the updater itself, as the SWIG binding's
      // PwMaterial<T>* results do (src/pw_material.hh:60-74)
      .def("attach",
           [](C& self, py::handle idx, const PwMaterialParam& p) -> C& {
             const auto v = as_index(idx);
             try {
               static_cast<PwMaterial<T>&>(self).attach(v.data(), static_cast<int>(v.size()), &p);
             } catch (const std::invalid_argument& e) {
               throw py::value_error(e.what());
             }
             return self;
           }, py::return_value_policy::reference)
      .def("merge", [](C& self, const C& other) -> C& {
        static_cast<PwMaterial<T>&>(self).merge(&other);
        return self;
      }, py::return_value_policy::reference)
      .def("update_all",
           [](C& self, py::array inplace, py::array in1, py::array in2, double d1,
              double d2, double dt, double n) {
             auto f0 = as_field<T>(inplace, true);
             auto f1 = as_field<T>(in1, false);
             auto f2 = as_field<T>(in2, false);
             if (!self.indices_in_bounds(f0.d1, f0.d2, f0.d3))
               throw py::index_error("field index is out of bounds");
             try {
               static_cast<PwMaterial<T>&>(self).update_all(f0.data, f0.d1, f0.d2, f0.d3, f1.data, f1.d1, f1.d2,
                               f1.d3, f2.data, f2.d1, f2.d2, f2.d3, d1, d2, dt, n);
             } catch (const std::invalid_argument& e) {
               throw py::value_error(e.what());
             } catch (const std::out_of_range& e) {
               throw py::index_error(e.what());
             }
           })
      .def("idx_size", &C::idx_size)
      .def("name", [](const C& self) { return self.name(); });
}

template <typename T, template <typename> class U>
void def_electric(py::module_& m, const std::string& name) {
  py::class_<U<T>, MaterialElectric<T>> cls(m, name.c_str());
  def_updater_methods<T>(cls);
  cls.def("get_eps_inf", [](const U<T>& self, py::handle idx) {
    const auto v = as_index(idx);
    return self.get_eps_inf(v.data(), static_cast<int>(v.size()));
  });
}

template <typename T, template <typename> class U>
void def_magnetic(py::module_& m, const std::string& name) {
  py::class_<U<T>, MaterialMagnetic<T>> cls(m, name.c_str());
  def_updater_methods<T>(cls);
  cls.def("get_mu_inf", [](const U<T>& self, py::handle idx) {
    const auto v = as_index(idx);
    return self.get_mu_inf(v.data(), static_cast<int>(v.size()));
  });
}

std::vector<std::array<double, 3>> rows3(py::array_t<double, py::array::c_style> a,
                                         const char* what) {
  if (a.ndim() != 2 || a.shape(1) != 3) throw py::value_error(what);
  std::vector<std::array<double, 3>> out(a.shape(0));
  for (py::ssize_t i = 0; i < a.shape(0); ++i)
    for (int j = 0; j < 3; ++j) out[i][j] = a.at(i, j);
  return out;
}

template <typename T>
void bind_all(py::module_& m, const std::string& sfx) {
  py::class_<ElectricParam<T>, PwMaterialParam>(m, ("ElectricParam" + sfx).c_str())
      .def_readwrite("eps_inf", &ElectricParam<T>::eps_inf);
  py::class_<MagneticParam<T>, PwMaterialParam>(m, ("MagneticParam" + sfx).c_str())
      .def_readwrite("mu_inf", &MagneticParam<T>::mu_inf);
  py::class_<PwMaterial<T>>(m, ("PwMaterial" + sfx).c_str());
  py::class_<MaterialElectric<T>, PwMaterial<T>>(m, ("MaterialElectric" + sfx).c_str());
  py::class_<MaterialMagnetic<T>, PwMaterial<T>>(m, ("MaterialMagnetic" + sfx).c_str());

  // Dummy
  py::class_<DummyElectricParam<T>, ElectricParam<T>>(m, ("DummyElectricParam" + sfx).c_str())
      .def(py::init<>());
  py::class_<DummyMagneticParam<T>, MagneticParam<T>>(m, ("DummyMagneticParam" + sfx).c_str())
      .def(py::init<>());
  def_electric<T, DummyEx>(m, "DummyEx" + sfx);
  def_electric<T, DummyEy>(m, "DummyEy" + sfx);
  def_electric<T, DummyEz>(m, "DummyEz" + sfx);
  def_magnetic<T, DummyHx>(m, "DummyHx" + sfx);
  def_magnetic<T, DummyHy>(m, "DummyHy" + sfx);
  def_magnetic<T, DummyHz>(m, "DummyHz" + sfx);

  // Const
  py::class_<ConstElectricParam<T>, ElectricParam<T>>(m, ("ConstElectricParam" + sfx).c_str())
      .def(py::init<>())
      .def_readwrite("value", &ConstElectricParam<T>::value);
  py::class_<ConstMagneticParam<T>, MagneticParam<T>>(m, ("ConstMagneticParam" + sfx).c_str())
      .def(py::init<>())
      .def_readwrite("value", &ConstMagneticParam<T>::value);
  def_electric<T, ConstEx>(m, "ConstEx" + sfx);
  def_electric<T, ConstEy>(m, "ConstEy" + sfx);
  def_electric<T, ConstEz>(m, "ConstEz" + sfx);
  def_magnetic<T, ConstHx>(m, "ConstHx" + sfx);
  def_magnetic<T, ConstHy>(m, "ConstHy" + sfx);
  def_magnetic<T, ConstHz>(m, "ConstHz" + sfx);

  // Dielectric
  py::class_<DielectricElectricParam<T>, ElectricParam<T>>(
      m, ("DielectricElectricParam" + sfx).c_str())
      .def(py::init<>());
  py::class_<DielectricMagneticParam<T>, MagneticParam<T>>(
      m, ("DielectricMagneticParam" + sfx).c_str())
      .def(py::init<>());
  def_electric<T, DielectricEx>(m, "DielectricEx" + sfx);
  def_electric<T, DielectricEy>(m, "DielectricEy" + sfx);
  def_electric<T, DielectricEz>(m, "DielectricEz" + sfx);
  def_magnetic<T, DielectricHx>(m, "DielectricHx" + sfx);
  def_magnetic<T, DielectricHy>(m, "DielectricHy" + sfx);
  def_magnetic<T, DielectricHz>(m, "DielectricHz" + sfx);

  // UPML
  py::class_<UpmlElectricParam<T>, ElectricParam<T>>(m, ("UpmlElectricParam" + sfx).c_str())
      .def(py::init<>())
      .def_readwrite("c1", &UpmlElectricParam<T>::c1)
      .def_readwrite("c2", &UpmlElectricParam<T>::c2)
      .def_readwrite("c3", &UpmlElectricParam<T>::c3)
      .def_readwrite("c4", &UpmlElectricParam<T>::c4)
      .def_readwrite("c5", &UpmlElectricParam<T>::c5)
      .def_readwrite("c6", &UpmlElectricParam<T>::c6)
      .def_readwrite("d", &UpmlElectricParam<T>::d);
  py::class_<UpmlMagneticParam<T>, MagneticParam<T>>(m, ("UpmlMagneticParam" + sfx).c_str())
      .def(py::init<>())
      .def_readwrite("c1", &UpmlMagneticParam<T>::c1)
      .def_readwrite("c2", &UpmlMagneticParam<T>::c2)
      .def_readwrite("c3", &UpmlMagneticParam<T>::c3)
      .def_readwrite("c4", &UpmlMagneticParam<T>::c4)
      .def_readwrite("c5", &UpmlMagneticParam<T>::c5)
      .def_readwrite("c6", &UpmlMagneticParam<T>::c6)
      .def_readwrite("b", &UpmlMagneticParam<T>::b);
  def_electric<T, UpmlEx>(m, "UpmlEx" + sfx);
  def_electric<T, UpmlEy>(m, "UpmlEy" + sfx);
  def_electric<T, UpmlEz>(m, "UpmlEz" + sfx);
  def_magnetic<T, UpmlHx>(m, "UpmlHx" + sfx);
  def_magnetic<T, UpmlHy>(m, "UpmlHy" + sfx);
  def_magnetic<T, UpmlHz>(m, "UpmlHz" + sfx);

  // CPML
  py::class_<CpmlElectricParam<T>, ElectricParam<T>>(m, ("CpmlElectricParam" + sfx).c_str())
      .def(py::init<>())
      .def_readwrite("b1", &CpmlElectricParam<T>::b1)
      .def_readwrite("b2", &CpmlElectricParam<T>::b2)
      .def_readwrite("c1", &CpmlElectricParam<T>::c1)
      .def_readwrite("c2", &CpmlElectricParam<T>::c2)
      .def_readwrite("kappa1", &CpmlElectricParam<T>::kappa1)
      .def_readwrite("kappa2", &CpmlElectricParam<T>::kappa2)
      .def_readwrite("psi1", &CpmlElectricParam<T>::psi1)
      .def_readwrite("psi2", &CpmlElectricParam<T>::psi2);
  py::class_<CpmlMagneticParam<T>, MagneticParam<T>>(m, ("CpmlMagneticParam" + sfx).c_str())
      .def(py::init<>())
      .def_readwrite("b1", &CpmlMagneticParam<T>::b1)
      .def_readwrite("b2", &CpmlMagneticParam<T>::b2)
      .def_readwrite("c1", &CpmlMagneticParam<T>::c1)
      .def_readwrite("c2", &CpmlMagneticParam<T>::c2)
      .def_readwrite("kappa1", &CpmlMagneticParam<T>::kappa1)
      .def_readwrite("kappa2", &CpmlMagneticParam<T>::kappa2)
      .def_readwrite("psi1", &CpmlMagneticParam<T>::psi1)
      .def_readwrite("psi2", &CpmlMagneticParam<T>::psi2);
  def_electric<T, CpmlEx>(m, "CpmlEx" + sfx);
  def_electric<T, CpmlEy>(m, "CpmlEy" + sfx);
  def_electric<T, CpmlEz>(m, "CpmlEz" + sfx);
  def_magnetic<T, CpmlHx>(m, "CpmlHx" + sfx);
  def_magnetic<T, CpmlHy>(m, "CpmlHy" + sfx);
  def_magnetic<T, CpmlHz>(m, "CpmlHz" + sfx);

  // Drude
  py::class_<DrudeElectricParam<T>, ElectricParam<T>>(m, ("DrudeElectricParam" + sfx).c_str())
      .def(py::init<>())
      .def("set", [](DrudeElectricParam<T>& p, py::array_t<double, py::array::c_style> a,
                     py::array_t<double, py::array::c_style> c) {
        if (a.ndim() != 2 || a.shape(1) != 3 || c.ndim() != 1 || c.shape(0) != 3)
          throw py::value_error("Drude coefficients require shapes (n, 3) and (3,)");
        for (auto& r : rows3(a, "bad a")) p.a.push_back(r);
        for (int i = 0; i < 3; ++i) p.c[i] = c.at(i);
        p.q_now.resize(a.shape(0), T(0));
        p.q_new.resize(a.shape(0), T(0));
      });
  py::class_<DrudeMagneticParam<T>, MagneticParam<T>>(m, ("DrudeMagneticParam" + sfx).c_str())
      .def(py::init<>());
  def_electric<T, DrudeEx>(m, "DrudeEx" + sfx);
  def_electric<T, DrudeEy>(m, "DrudeEy" + sfx);
  def_electric<T, DrudeEz>(m, "DrudeEz" + sfx);
  def_magnetic<T, DrudeHx>(m, "DrudeHx" + sfx);
  def_magnetic<T, DrudeHy>(m, "DrudeHy" + sfx);
  def_magnetic<T, DrudeHz>(m, "DrudeHz" + sfx);

  // Lorentz
  py::class_<LorentzElectricParam<T>, ElectricParam<T>>(
      m, ("LorentzElectricParam" + sfx).c_str())
      .def(py::init<>())
      .def("set", [](LorentzElectricParam<T>& p, py::array_t<double, py::array::c_style> a,
                     py::array_t<double, py::array::c_style> c) {
        if (a.ndim() != 2 || a.shape(1) != 3 || c.ndim() != 1 || c.shape(0) != 3)
          throw py::value_error("Lorentz coefficients require shapes (n, 3) and (3,)");
        for (auto& r : rows3(a, "bad a")) p.a.push_back(r);
        for (int i = 0; i < 3; ++i) p.c[i] = c.at(i);
        p.l_now.resize(a.shape(0));
        p.l_new.resize(a.shape(0));
      });
  py::class_<LorentzMagneticParam<T>, MagneticParam<T>>(
      m, ("LorentzMagneticParam" + sfx).c_str())
      .def(py::init<>());
  def_electric<T, LorentzEx>(m, "LorentzEx" + sfx);
  def_electric<T, LorentzEy>(m, "LorentzEy" + sfx);
  def_electric<T, LorentzEz>(m, "LorentzEz" + sfx);
  def_magnetic<T, LorentzHx>(m, "LorentzHx" + sfx);
  def_magnetic<T, LorentzHy>(m, "LorentzHy" + sfx);
  def_magnetic<T, LorentzHz>(m, "LorentzHz" + sfx);

  // Drude-critical points, ADE form
  py::class_<DcpAdeElectricParam<T>, ElectricParam<T>>(
      m, ("DcpAdeElectricParam" + sfx).c_str())
      .def(py::init<>())
      .def("set", [](DcpAdeElectricParam<T>& p, py::array_t<double, py::array::c_style> a,
                     py::array_t<double, py::array::c_style> b,
                     py::array_t<double, py::array::c_style> c) {
        if (a.ndim() != 2 || a.shape(1) != 3 || b.ndim() != 2 || b.shape(1) != 5 ||
            c.ndim() != 1 || c.shape(0) != 4)
          throw py::value_error(
              "DcpAde coefficients require shapes (n, 3), (n, 5), and (4,)");
        for (auto& r : rows3(a, "bad a")) p.a.push_back(r);
        for (py::ssize_t i = 0; i < b.shape(0); ++i) {
          std::array<double, 5> r;
          for (int j = 0; j < 5; ++j) r[j] = b.at(i, j);
          p.b.push_back(r);
        }
        for (int i = 0; i < 4; ++i) p.c[i] = c.at(i);
        p.q_old.resize(a.shape(0));
        p.q_now.resize(a.shape(0));
        p.p_old.resize(b.shape(0));
        p.p_now.resize(b.shape(0));
      });
  py::class_<DcpAdeMagneticParam<T>, MagneticParam<T>>(
      m, ("DcpAdeMagneticParam" + sfx).c_str())
      .def(py::init<>());
  def_electric<T, DcpAdeEx>(m, "DcpAdeEx" + sfx);
  def_electric<T, DcpAdeEy>(m, "DcpAdeEy" + sfx);
  def_electric<T, DcpAdeEz>(m, "DcpAdeEz" + sfx);
  def_magnetic<T, DcpAdeHx>(m, "DcpAdeHx" + sfx);
  def_magnetic<T, DcpAdeHy>(m, "DcpAdeHy" + sfx);
  def_magnetic<T, DcpAdeHz>(m, "DcpAdeHz" + sfx);

  // Drude-critical points, PLRC form (DcpRc uses it with other coefficients)
  py::class_<DcpPlrcElectricParam<T>, ElectricParam<T>>(
      m, ("DcpPlrcElectricParam" + sfx).c_str())
      .def(py::init<>())
      .def("set", [](DcpPlrcElectricParam<T>& p, py::array_t<double, py::array::c_style> a,
                     py::array_t<std::complex<double>, py::array::c_style> b,
                     py::array_t<double, py::array::c_style> c) {
        if (a.ndim() != 2 || a.shape(1) != 3 || b.ndim() != 2 || b.shape(1) != 3 ||
            c.ndim() != 1 || c.shape(0) != 3)
          throw py::value_error(
              "DcpPlrc coefficients require shapes (n, 3), (n, 3), and (3,)");
        for (auto& r : rows3(a, "bad a")) p.a.push_back(r);
        for (py::ssize_t i = 0; i < b.shape(0); ++i) {
          std::array<std::complex<double>, 3> r;
          for (int j = 0; j < 3; ++j) r[j] = b.at(i, j);
          p.b.push_back(r);
        }
        for (int i = 0; i < 3; ++i) p.c[i] = c.at(i);
        p.psi_dp_re.resize(a.shape(0));
        p.psi_dp_im.resize(a.shape(0));
        p.psi_cp_re.resize(b.shape(0));
        p.psi_cp_im.resize(b.shape(0));
      });
  py::class_<DcpPlrcMagneticParam<T>, MagneticParam<T>>(
      m, ("DcpPlrcMagneticParam" + sfx).c_str())
      .def(py::init<>());
  def_electric<T, DcpPlrcEx>(m, "DcpPlrcEx" + sfx);
  def_electric<T, DcpPlrcEy>(m, "DcpPlrcEy" + sfx);
  def_electric<T, DcpPlrcEz>(m, "DcpPlrcEz" + sfx);
  def_magnetic<T, DcpPlrcHx>(m, "DcpPlrcHx" + sfx);
  def_magnetic<T, DcpPlrcHy>(m, "DcpPlrcHy" + sfx);
  def_magnetic<T, DcpPlrcHz>(m, "DcpPlrcHz" + sfx);
}

}  // namespace

PYBIND11_MODULE(pw_material, m) {
  py::class_<PwMaterialParam>(m, "PwMaterialParam");
  bind_all<double>(m, "Real");
  bind_all<std::complex<double>>(m, "Cmplx");
  m.def("openmp_enabled", &openmp_enabled);
  m.def("openmp_max_threads", &openmp_max_threads);
  m.def("openmp_cell_threshold", &openmp_cell_threshold);
}
