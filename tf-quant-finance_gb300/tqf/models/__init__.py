"""Models namespace (tff/models/__init__.py:17-45): the SDE path-simulation API."""

from tqf.models import coefficients  # noqa: F401
from tqf.models import euler_sampling  # noqa: F401
from tqf.models import hjm  # noqa: F401
from tqf.models import hull_white  # noqa: F401
from tqf.models import longstaff_schwartz  # noqa: F401
from tqf.models import milstein_sampling  # noqa: F401
from tqf.models import utils  # noqa: F401
from tqf.models.generic_ito_process import GenericItoProcess  # noqa: F401
from tqf.models.geometric_brownian_motion import GeometricBrownianMotion  # noqa: F401
from tqf.models.heston_model import HestonModel  # noqa: F401
from tqf.models.ito_process import ItoProcess  # noqa: F401
from tqf.models.multivariate_gbm import MultivariateGeometricBrownianMotion  # noqa: F401

__all__ = ["coefficients", "euler_sampling", "hjm", "hull_white", "longstaff_schwartz", "milstein_sampling", "GeometricBrownianMotion", "utils", "GenericItoProcess", "HestonModel", "ItoProcess",
           "MultivariateGeometricBrownianMotion"]
