"""ctypes mirror of include/fdtd_gb300.h (descriptor structs and constants)."""
import ctypes as C

FDTD_OK, FDTD_EINVAL, FDTD_ENOMEM, FDTD_ECUDA, FDTD_ESTATE, FDTD_ERANGE, FDTD_ENODEV = range(7)

LAYOUT_1D, LAYOUT_2D_TE, LAYOUT_2D_TM, LAYOUT_3D = 1, 2, 3, 4
F32, F64 = 1, 2
EX, EY, EZ, HX, HY, HZ, EX_INC, HZ_INC = range(8)
COMP_NAMES = {"Ex": EX, "Ey": EY, "Ez": EZ, "Hx": HX, "Hy": HY, "Hz": HZ,
              "Ex_inc": EX_INC, "Hz_inc": HZ_INC}
REGION_BOX, REGION_SPHERES, REGION_MASK = 0, 1, 2
PML_REFERENCE, PML_SPLIT = 1, 2
KERNEL_E, KERNEL_H, KERNEL_DFT, KERNEL_LINE1D, KERNEL_EDGE, KERNEL_ADE, KERNEL_STEP, KERNEL_COUNT = range(8)

I3 = C.c_int32 * 3


class GridDesc(C.Structure):
    _fields_ = [("layout", C.c_int32), ("precision", C.c_int32), ("n", I3),
                ("periodic", I3), ("main_lo", I3), ("main_hi", I3),
                ("ku", C.c_double), ("dt", C.c_double), ("ds", C.c_double)]


class Region(C.Structure):
    _fields_ = [("kind", C.c_int32), ("lo", I3), ("hi", I3), ("count", C.c_int32),
                ("centers_radii", C.POINTER(C.c_double)), ("mask", C.POINTER(C.c_uint8))]


class Drude2CP(C.Structure):
    _fields_ = [("eps_inf", C.c_double), ("omega_d", C.c_double), ("gamma_d", C.c_double),
                ("amp", C.c_double * 2), ("phi", C.c_double * 2),
                ("omega", C.c_double * 2), ("gamma", C.c_double * 2)]


class GrapheneDesc(C.Structure):
    _fields_ = [("fermi_ev", C.c_double), ("tau", C.c_double), ("temperature", C.c_double),
                ("chi3", C.c_double), ("raman_frac", C.c_double), ("raman_freq", C.c_double),
                ("raman_tau", C.c_double), ("thickness", C.c_double), ("e_scale", C.c_double)]


class TfsfDesc(C.Structure):
    _fields_ = [("lo", I3), ("hi", I3), ("eps_line", C.c_double)]


E_INC, H_INC = 6, 7
LORENTZ_JP, LORENTZ_S = 0, 1
LORENTZ_MAX_POLES = 4


class LorentzDesc(C.Structure):
    _fields_ = [("form", C.c_int32), ("npoles", C.c_int32), ("eps_inf", C.c_double),
                ("delta_eps", C.c_double * LORENTZ_MAX_POLES), ("omega", C.c_double * LORENTZ_MAX_POLES),
                ("gamma", C.c_double * LORENTZ_MAX_POLES), ("sheet", C.c_int32), ("ez_uses_x_current", C.c_int32),
                ("chi3", C.c_double), ("w_nl", C.c_double), ("gamma_nl", C.c_double), ("e_scale", C.c_double)]


RAMAN_EXACT, RAMAN_CENTRAL = 0, 1


class GrapheneNkDesc(C.Structure):
    _fields_ = [("n", C.c_double), ("k", C.c_double), ("wavelength", C.c_double), ("scale", C.c_double),
                ("chi3", C.c_double), ("alpha", C.c_double), ("w_nl", C.c_double), ("gamma_nl", C.c_double)]


class GrapheneCpDesc(C.Structure):
    _fields_ = [("eps_inf", C.c_double), ("drude_omega", C.c_double), ("drude_gamma", C.c_double),
                ("amp", C.c_double * 4), ("phi", C.c_double * 4), ("omega", C.c_double * 4),
                ("gamma", C.c_double * 4), ("width", C.c_double), ("chi3", C.c_double),
                ("w_nl", C.c_double), ("gamma_nl", C.c_double), ("raman_form", C.c_int32),
                ("normal_axis", C.c_int32)]


class PmlDesc(C.Structure):
    _fields_ = [("mode", C.c_int32), ("npml", (C.c_int32 * 2) * 3),
                ("eps_lo", C.c_double), ("eps_hi", C.c_double),
                ("sigma_max", C.c_double), ("order", C.c_double)]


class SourceDesc(C.Structure):
    _fields_ = [("component", C.c_int32), ("lo", I3), ("hi", I3), ("amp", C.c_double),
                ("t0", C.c_double), ("st", C.c_double), ("w0", C.c_double)]


class MonitorDesc(C.Structure):
    _fields_ = [("lo", I3), ("hi", I3), ("comp_mask", C.c_int32),
                ("n_first", C.c_int32), ("n_last", C.c_int32), ("nfreq", C.c_int32),
                ("omega", C.POINTER(C.c_double)), ("reduce", C.c_int32)]


class ProbeDesc(C.Structure):
    _fields_ = [("cell", I3), ("comp_mask", C.c_int32),
                ("n_first", C.c_int32), ("n_last", C.c_int32)]


class Tfsf1dDesc(C.Structure):
    _fields_ = [("boundary", C.c_int32), ("eps_lo", C.c_double), ("eps_hi", C.c_double)]


class ServerDesc(C.Structure):
    _fields_ = [("hbm_budget", C.c_uint64), ("max_active", C.c_int32), ("chunk_steps", C.c_int32),
                ("pack_cells", C.c_int32)]


class ServerStatus(C.Structure):
    _fields_ = [("queued", C.c_int32), ("active", C.c_int32), ("finished", C.c_int64),
                ("held_bytes", C.c_uint64), ("held_bytes_max", C.c_uint64), ("budget_bytes", C.c_uint64),
                ("packed_rings", C.c_int64), ("pack_builds", C.c_int64), ("pack_build_s", C.c_double)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = range(4)

MONITOR_CELLS, MONITOR_MEAN = 0, 1
