"""tqf — GB300-native (sm_103a) Monte Carlo engine behind tf-quant-finance's
SDE path-simulation API.

Drop-in entry points (same signatures as the reference):

* ``tqf.models.euler_sampling.sample`` / ``tqf.models.GenericItoProcess``
  (tff/models/euler_sampling.py:27, tff/models/generic_ito_process.py:187)
* ``tqf.models.HestonModel`` (tff/models/heston/heston_model.py:38)
* ``tqf.math.random.sobol.sample`` (tff/math/random_ops/sobol/sobol_impl.py:39)

Results are torch tensors on the current CUDA device; all compute runs in the
hand-written kernels of libtqf.so.
"""

from tqf import math  # noqa: F401
from tqf import models  # noqa: F401
from tqf import pricing  # noqa: F401
from tqf.errors import InvalidArgumentError  # noqa: F401

__all__ = ["math", "models", "pricing", "InvalidArgumentError"]
