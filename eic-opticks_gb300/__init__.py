"""eic-opticks_gb300 : GB300-native optical-photon transport engine (host-side Python mirror).

The engine itself is native: CUDA kernels and the C ABI in ``csrc/`` build into ``libgbopticks.so``.  This package
holds what sits around it on the host:

* ``layout``    numpy dtypes of the reference array layouts (sphoton, quad6, CSGNode, ...)
* ``geometry``  CSGFoundry-layout geometry and boundary tables for the benchmark geometries
* ``gensteps``  genstep / input-photon producers
* ``engine``    ctypes binding of the C ABI with a ``G4CXOpticks``-shaped facade
* ``build``     compile recipe for the CUDA library (sm_103a)
"""
from . import layout, geometry, gensteps  # noqa: F401
