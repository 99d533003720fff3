// Stand-in for pybind11/eigen.h when building the reference's py_rccsd
// module from its sources. Test infrastructure only.
//
// The reference includes this header (src/py_rccsd.cpp:1) but binds no
// Eigen type, and Eigen is an empty submodule in the reference checkout,
// so an empty header is all the build needs.
#pragma once
