"""GB300-native per-timestep simulation cycle of synaptogenesis.

The product is the C-ABI shared library built from ``csrc/`` (see
``include/syngen.h``); ``syngen`` is its Python front-end with the reference's
API.  ``build.build()`` compiles the library for sm_103a.
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsyngen.so")


def lib_path():
    """Path of the in-tree library; raises if it has not been built."""
    if not os.path.exists(LIB_PATH):
        raise ImportError("libsyngen.so not built; run synaptogenesis_gb300.build.build()")
    return LIB_PATH
