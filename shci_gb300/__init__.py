"""GB300-native SHCI hot path: heat-bath selection, Hamiltonian build, Davidson and PT2 on
one GPU behind the C ABI of include/shci_gpu.h (libshci_gpu.so)."""
from ._lib import Context, ShciError, PREC_FP64, PREC_MIXED, load  # noqa: F401
