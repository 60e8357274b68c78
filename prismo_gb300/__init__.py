"""GB300-native (sm_103a) FDTD time stepping behind Prismo's backend interface.

The compute path is ``libprismo_cuda.so`` (hand-written CUDA, C ABI in
include/prismo_cuda.h) driven through ctypes; PyTorch provides device memory
and streams.  There is no CPU fallback: operations raise when the native
library or a CUDA device is missing.
"""

__version__ = "0.1.0"

from .grid import GridSpec, YeeGrid  # noqa: F401,E402
from .pml import PMLParams  # noqa: F401,E402
from .sources import (  # noqa: F401,E402
    ContinuousWave,
    CustomWaveform,
    ElectricDipole,
    GaussianBeamSource,
    GaussianPulse,
    LineSource,
    MagneticDipole,
    ModeSource,
    PlaneWaveSource,
    PointSource,
    Source,
    TFSFSource,
    Waveform,
)
from .backend import CudaBackend, DeviceArray, get_backend, get_backend_info, list_available_backends, set_backend  # noqa
from .fields import ElectromagneticFields  # noqa: F401,E402
from .materials import (  # noqa: F401,E402
    DebyeMaterial,
    DrudeLorentzMaterial,
    DrudeMaterial,
    LorentzMaterial,
    LorentzPole,
)
from .monitors import DFTMonitor, FieldMonitor, FluxMonitor, ModeExpansionMonitor, Monitor  # noqa: F401,E402
from . import export  # noqa: F401,E402
from .tensor import AnisotropicUpdater, TensorComponents, TensorMaterial  # noqa: F401,E402
from .ports import ModePort, ModePortConfig  # noqa: F401,E402
from .simulation import Simulation  # noqa: F401,E402
from .solver import FDTDSolver, MaxwellUpdater  # noqa: F401,E402
