"""GB300 backend for SNNCuda's per-tick spiking simulation path.

The compute path is hand-written CUDA for sm_103a in `csrc/`, built into
`_lib/libsnncuda_gb300.so` behind the C ABI of include/snncuda_gb300.h.
This package holds the host-side mirror of the reference interface.
"""

from .connectome import (AMPA, APICAL, BASAL, GABA_A, GABA_B, INHIBITORY, NMDA, SOMA, Connectome,
                         ExplicitConnection, NetworkBuilder, NeuronParams, Projection)
from .simulation import (BACKEND_LIBRARY, Batch, NetworkPropagator, SNNCudaError, Server, Simulation, backend,
                         default_config)
from .declarative import load as load_network


def version() -> str:
    """snncuda_version() of the backend library (SNNCudaC.h:7)."""
    return backend().snncuda_version().decode("utf-8")


def cuda_available() -> bool:
    """snncuda_cuda_available() of the backend library (SNNCudaC.h:8)."""
    return bool(backend().snncuda_cuda_available())


__all__ = [
    "AMPA", "APICAL", "BASAL", "GABA_A", "GABA_B", "INHIBITORY", "NMDA", "SOMA", "Connectome",
    "ExplicitConnection", "NetworkBuilder", "NeuronParams", "Projection", "BACKEND_LIBRARY",
    "Batch", "NetworkPropagator", "SNNCudaError", "Server", "Simulation", "backend", "default_config", "version",
    "cuda_available", "load_network",
]
