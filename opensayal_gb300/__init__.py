"""GB300-native drop-in for OpenSayal's wind-tunnel simulation step.

The compute path is libopensayal_gb300.so (hand-written sm_103a CUDA behind the
C ABI in include/opensayal_gb300.h); this package builds and binds it.
"""
from .build import build_library, LIB_PATH
from .fluid import CONFIG_KEYS, Fluid, Source, default_config, load_config
from .native import OsConfig, OsSource, NativeError

__all__ = [
    "build_library", "LIB_PATH", "Fluid", "Source", "default_config", "load_config",
    "CONFIG_KEYS", "OsConfig", "OsSource", "NativeError",
]
