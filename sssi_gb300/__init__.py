"""sssi_gb300 -- SSSI's finite-difference core (acoustic CPML and sponge, elastic SPML) on GB300 (sm_103a).

Host side of the drop-in: the MATLAB-shaped functions in :mod:`sssi_gb300.api`
call the C ABI of ``libsssi_gb300.so`` (``include/sssi_gb300.h``), whose
kernels are hand-written CUDA for sm_103a.  Import never touches the GPU;
the first call loads the library and fails loudly if it is not built.
"""
from .api import (  # noqa: F401
    MODES,
    Plan,
    dampPml,
    debug_divide,
    debug_schedule3d,
    debug_tile_shape,
    debug_withhold_copy,
    dCoef,
    diffOperator,
    enable_timing,
    last_timing,
    fwdTimeCpmlFor2dAw,
    fwdTimeCpmlFor2dAwPoint,
    fwdTimeCpmlFor3dAw,
    fwdTimeCpmlFor3dAwPoint,
    fwdTimeSpmlFor2dEw,
    fwdTimeSpmlFor2dEwPoint,
    fwdTimeSpmlFor3dEw,
    fwdTimeSpmlFor3dEwPoint,
    fwdTimeSpongeFor2dAw,
    fwdTimeSpongeFor2dAwPoint,
    launch_count,
    mat_read,
    mat_write,
    measure_fp64_rate,
    release_cache,
    rtmTimeCpmlFor2dAw,
    rtmTimeSpongeFor2dAw,
    rvsTimeCpmlFor2dAw,
    rvsTimeSpongeFor2dAw,
    set_stream,
)
from ._native import SSSIError  # noqa: F401

__version__ = "0.1.0"
