"""GB300-native direct-SCF Fock builder (drop-in for the ERI/Fock path of
lyuhang428/SegFault_py, src/hf).

The compute path is libsegfock.so (sm_103a CUDA kernels behind a C ABI,
include/segfock.h); this package is the Python host side: basis/molecule
ingestion, the ctypes binding, the Fock builder and the SCF drivers.
"""
import os as _os

# The Fock build forks its launches onto 16 streams; with CUDA's default of 8
# hardware work queues pairs of streams share a queue and a launch waits
# behind another stream's.  The variable is read when the CUDA context is
# created, so it only applies when this package is imported before CUDA is
# first used; a value set by the user is kept.
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "16")

from .molecule import Atom, BasisSetNotAvailableError, ContractedGaussianFunction, Molecule  # noqa: F401

__all__ = ["Molecule", "Atom", "ContractedGaussianFunction", "BasisSetNotAvailableError",
           "FockBuilder", "eri_rys", "scf", "scf_damping", "scf_diis"]


def __getattr__(name):
    if name in ("FockBuilder", "eri_rys"):
        from . import fock
        return getattr(fock, name)
    if name in ("scf", "scf_damping", "scf_diis", "SCFResult"):
        from . import scf as _scf
        return getattr(_scf, name)
    raise AttributeError(name)
