"""GB300-native LASSIE integrator (mass-action ODEs, RKF45 -> backward-Euler
Newton) with a drop-in CLI and a C ABI over sm_103a CUDA kernels."""
from .model import Model, CompiledModel, compile_model, load_folder, write_folder  # noqa: F401

__version__ = "0.1.0"
