"""GB300-native range-sensor ray casting with rmagine's simulator interface.

Compute runs in librmg_gb300.so (hand-written sm_103a kernels behind the C
ABI of include/rmg.h); this package is the Python host layer over that ABI.
"""
from ._lib import RmgError, load  # noqa: F401
from .sensors import (DiscreteInterval, Interval, O1DnModel, OnDnModel, PinholeModel,  # noqa: F401
                      SphericalModel, depth_camera, example_o1dn, example_ondn, example_pinhole,
                      example_spherical, ouster_like, vlp16_360, vlp16_900)
from .simulation import (ATTRIBUTES, Bundle, Instance, IntAttrAll, Map, O1DnSimulator,  # noqa: F401
                         OnDnSimulator, PinholeSimulator, Scene, Sensor, SphereSimulator,
                         identity_transforms, launch_config, make_simulator, make_transforms,
                         resize_memory_bundle)

__version__ = "0.1.0"
