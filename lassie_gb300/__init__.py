"""GB300-native LASSIE integrator (mass-action ODEs, RKF45 -> backward-Euler
Newton) with a drop-in CLI and a C ABI over sm_103a CUDA kernels.

Entry points (``lassie_gb300.solver``):

* ``simulate(model)`` / ``simulate_batch(models)`` / ``Batch(models)``:
  LASSIE's own step control, mixed (FP32 factors, FP64 refinement) or FP64;
  ``bdf={"rtol": ..., "atol": ...}`` selects the variable-order BDF
  controller with rtol/atol error control instead.
* ``rhs``, ``newton_matrix``: single evaluations (the C ABI also has batched
  device-buffer forms, ``lassie_rhs_device`` and
  ``lassie_newton_matrix_device``).

``lassie_gb300.adjoint`` has the discrete adjoint (d loss / d log k) behind a
``torch.autograd.Function`` and a parameter-fit loop; ``lassie_gb300.sbml``
reads and writes SBML mass-action models.
"""
from .model import Model, CompiledModel, compile_model, load_folder, write_folder  # noqa: F401

__version__ = "0.1.0"
