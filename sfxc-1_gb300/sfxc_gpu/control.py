"""The correlation set-up of a control file and a VEX file (sfxc_gpu_control_*):
Control_parameters' derivations and the manager's dealing of the jobs
(sfxc/src/control_parameters.cc, sfxc/src/manager_node.cc), computed by the
library and returned as a dict."""
import ctypes as C
import json

from . import lib as L


def plan(ctrl_path, vex_path, station_time=None):
    """The plan of a correlation.  station_time(station, scan) -> ticks, if
    given, is the input node's current time when the manager starts that scan
    (control-file station index, plan scan index).  Raises SfxcError when the
    files cannot be read or the set-up is refused."""
    lib = L.load()
    h = lib.sfxc_gpu_control_open(str(ctrl_path).encode(), str(vex_path).encode())
    if not h:
        raise L.SfxcError(L.EINVAL, lib.sfxc_gpu_global_error().decode())
    try:
        err = []

        def cb(user, station, scan):
            try:
                return int(station_time(station, scan))
            except Exception as e:  # an exception cannot cross the C boundary
                err.append(e)
                return 0

        fn = L.STATION_TIME(cb) if station_time else L.STATION_TIME()
        n = lib.sfxc_gpu_control_plan(h, fn, None)
        if err:
            raise err[0]
        if n < 0:
            raise L.SfxcError(int(n), lib.sfxc_gpu_global_error().decode())
        return json.loads(lib.sfxc_gpu_control_plan_text(h).decode())
    finally:
        lib.sfxc_gpu_control_close(h)
