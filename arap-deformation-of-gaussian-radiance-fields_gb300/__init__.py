"""GB300 (sm_103a) embedded-deformation / ARAP hot path for Gaussian radiance
fields: kNN skinning weights, node graph, Gauss-Newton solve of node
transforms, and skinning of Gaussians and grid samples, behind the C ABI of
``include/arap_gb300.h`` (``libarap_gb300.so``)."""
from ._lib import ArapError, load  # noqa: F401

__version__ = "0.1.0"
