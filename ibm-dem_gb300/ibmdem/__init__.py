"""Host side of the GB300 IBM-DEM particle hot path.

`ibmdem.records` holds the C-ABI record layouts, `ibmdem.scenario` the seeded
synthetic cases, and `ibmdem.lib` / `ibmdem.api` the binding to the CUDA
library libibmdem.so (built by __graft_entry__.build()).  Importing this
package does not load the CUDA library; `ibmdem.api.Case` does, and raises if
it is missing.
"""
from . import records, scenario  # noqa: F401
