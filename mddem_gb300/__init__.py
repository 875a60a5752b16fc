"""mddem_gb300 -- GB300-native particle hot path of MDDEM (DEM + LJ) behind a C ABI.

The compute path is libmddem_gb300.so (hand-written CUDA for sm_103a); this
package holds its build recipe, the ctypes binding of include/mdg.h, the
reference-style configuration, the seeded input generators, restart files,
the benchmark workloads and the Python TOML runner.  The C++ host with the
reference's App / plugin shape is csrc/host (built into _lib/mdg_run).
"""
from .config import (ConfigError, Material, SimConfig, Wall, from_toml, granular_gas_config,  # noqa: F401
                     lj_fluid_config)

__all__ = ["ConfigError", "Material", "SimConfig", "Wall", "from_toml", "granular_gas_config", "lj_fluid_config"]
