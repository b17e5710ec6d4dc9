"""redgb: GB300 (sm_103a) implementation of red.cuda's hot path behind a C ABI.

Modules: `types` (record layouts), `bodies` (body-list files, synthetic disks), `api`
(the System view of one context), `lib` (loads libredgb.so), `driver` (the reference's
time loop with its output cadence), `build` (nvcc build of the library).
"""
from . import types  # noqa: F401
from .bodies import Disk, config_disk, make_disk, read_body_file, thresholds, write_body_file  # noqa: F401

__all__ = ["types", "Disk", "config_disk", "make_disk", "read_body_file", "write_body_file", "thresholds"]
