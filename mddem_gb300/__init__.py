"""mddem_gb300 -- GB300-native particle hot path of MDDEM (DEM + LJ) behind a C ABI.

The compute path is libmddem_gb300.so (hand-written CUDA for sm_103a); this
package holds its build recipe, the ctypes binding of include/mdg.h, the
reference-style configuration, the seeded input generators and the host-side
plugin layer.
"""
from .config import ConfigError, Material, SimConfig, from_toml, granular_gas_config, lj_fluid_config  # noqa: F401

__all__ = ["ConfigError", "Material", "SimConfig", "from_toml", "granular_gas_config", "lj_fluid_config"]
