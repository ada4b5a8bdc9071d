"""vnec_gb300: GB300-native VNEC mxv (SpMV) behind the OpenSparseBLAS C API.

* ``api``        — Python mirror of the reference interface over the C ABI.
* ``generators`` — seeded synthetic matrices (uniform-k, R-MAT, stencil, ...).
* ``mtxio``      — Matrix Market and GAP ``.sg`` readers.
* ``build``      — in-tree build of the native libraries.
"""
__all__ = ["api", "generators", "mtxio", "build"]
