"""GB300-native MTGP: bit-exact GPU drop-in for the MTGP reference C API.

The compute path is the CUDA library mtgp_gb300/lib/libmtgp_gb300.so
(kernels for sm_103a behind the C ABI of include/mtgp_gpu.h); this package
is its Python binding.  Build with `python -m mtgp_gb300.build`.
"""
from .params import MTGP32Params, MTGP64Params, load_table, jump_table, jump_string  # noqa: F401
