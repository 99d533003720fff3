"""fricc_gb300: the FRI-CCSD amplitude iteration of fri-cc on GB300 (sm_103a).

* ``fricc_gb300.py_rccsd`` -- drop-in for the reference's ``py_rccsd`` module
  (SparseTensor4d, contract_DTSpT) backed by the CUDA library;
* ``fricc_gb300.friccsd.FRICCSDGPU`` -- the whole iteration resident on the GPU;
* ``fricc_gb300.synthetic`` -- seeded synthetic systems (Cholesky ERIs, MP2 T2).

The CUDA library (libfricc_gb300.so, C ABI in include/fricc_gb300.h) is built
in-tree by ``fricc_gb300.build.build()``.
"""
__version__ = "0.1.0"
