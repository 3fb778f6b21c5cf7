"""ctypes binding of libmsmgb.so (include/msmgb.h).  Loading fails loudly when the library
is missing or was not built: there is no CPU fallback."""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmsmgb.so")

OK = 0
ERR_ARG, ERR_CUDA, ERR_NL_OVERFLOW, ERR_OUT_OF_BOX = -1, -2, -3, -4
ERR_RHO_RANGE, ERR_BOX_TOO_SMALL, ERR_NO_DEVICE, ERR_CAPACITY, ERR_TIMEOUT = -5, -6, -7, -8, -9
FS_TYPE, EAM_TYPE = 0, 1
PREC_FP64, PREC_MIXED, PREC_FF = 0, 1, 2
PRECISIONS = {"fp64": PREC_FP64, "mixed": PREC_MIXED, "ff": PREC_FF}
ORDER_ORIGINAL, ORDER_SORTED = 0, 1
LSPT_EACH_VR_FILE = 1
POT_CR, POT_MARINICA2, POT_ACKLAND_WW = 1, 2, 3
POT_DERLET_WW, POT_HEHE_EXP6, POT_HEW_ZBL = 4, 5, 6
POT_MARINICA3, POT_MARINICA4 = 7, 8
POT_AV_CU, POT_AV_AU, POT_AV_CUAU = 9, 10, 11
POT_MENDELEV_ZR = 12
POT_AWB_ZR = 13
POT_HETI_LJ = 14
STATU_ACTIVE = 1
STATU_FIXPOSX, STATU_FIXPOSY, STATU_FIXPOSZ = 2, 4, 8
STATU_FIXVELX, STATU_FIXVELY, STATU_FIXVELZ = 16, 32, 64
STATU_OUTOFBOX, STATU_REFLECT, STATU_TRANSMIT = 65536, 131072, 262144

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Params(C.Structure):
    _fields_ = [("device", C.c_int), ("max_atoms", C.c_int), ("max_boxes", C.c_int),
                ("mxkvois", C.c_int), ("rc_nl", C.c_double), ("skin_trigger", C.c_double),
                ("nb_uptab", C.c_int), ("precision", C.c_int), ("stream", C.c_void_p)]


class ForceTable(C.Structure):
    _fields_ = [("pottype", C.c_int), ("ntab", C.c_int), ("nkind", C.c_int),
                ("rmax", C.c_double), ("potr", _dp), ("fpotr", _dp), ("potb", _dp),
                ("fpotb", _dp), ("nembd", C.c_int), ("nkind1", C.c_int), ("rhod", C.c_double),
                ("fembd", _dp), ("dfembd", _dp), ("ngroup", C.c_int), ("kpair", _ip),
                ("kembd", _ip), ("ru", C.c_double)]


class Box(C.Structure):
    _fields_ = [("natom", C.c_int), ("lo", C.c_double * 3), ("len", C.c_double * 3),
                ("ifpd", C.c_int * 3)]


NOALLOC_MAX_ATOMS = 1048576
UNITS_EV_A, UNITS_CGS = 0, 1


class ForceNoAlloc(C.Structure):
    _fields_ = [("n", C.c_int), ("xp", C.c_void_p), ("statu", C.c_void_p), ("kvois", C.c_void_p),
                ("indi", C.c_void_p), ("ld", C.c_int), ("box_len", C.c_double * 3),
                ("ifpd", C.c_int * 3), ("pottype", C.c_int), ("ntab", C.c_int),
                ("rmax", C.c_double), ("ru", C.c_double), ("potb", C.c_void_p),
                ("fpotr", C.c_void_p), ("fpotb", C.c_void_p), ("nembd", C.c_int),
                ("rhod", C.c_double), ("dfembd", C.c_void_p), ("fp", C.c_void_p),
                ("stream", C.c_void_p), ("errbuf", C.c_char_p), ("errlen", C.c_int)]


class ExtForceView(C.Structure):
    _fields_ = [("n", C.c_int), ("nbox", C.c_int), ("stream", C.c_void_p), ("pos", C.c_void_p),
                ("fx", C.c_void_p), ("fy", C.c_void_p), ("fz", C.c_void_p), ("gid", C.c_void_p),
                ("ityp", C.c_void_p), ("statu", C.c_void_p), ("boxid", C.c_void_p)]


EXTFORCE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(ExtForceView))


# (name, restype, argtypes) of every exported entry point
SIGNATURES = [
    ("msmgb_create", C.c_int, [C.POINTER(C.c_void_p), C.POINTER(Params)]),
    ("msmgb_destroy", C.c_int, [C.c_void_p]),
    ("msmgb_last_error", C.c_char_p, [C.c_void_p]),
    ("msmgb_stream", C.c_void_p, [C.c_void_p]),
    ("msmgb_set_precision", C.c_int, [C.c_void_p, C.c_int]),
    ("msmgb_launch_count", C.c_int64, [C.c_void_p]),
    ("msmgb_synchronize", C.c_int, [C.c_void_p]),
    ("msmgb_init_forcetable", C.c_int, [C.c_void_p, C.POINTER(ForceTable)]),
    ("msmgb_clear_forcetable", C.c_int, [C.c_void_p]),
    ("msmgb_calforce", C.c_int, [C.c_void_p]),
    ("msmgb_calptensor", C.c_int, [C.c_void_p, _dp]),
    ("msmgb_calepot", C.c_int, [C.c_void_p]),
    ("msmgb_calden", C.c_int, [C.c_void_p]),
    ("msmgb_cal_atomic_stress", C.c_int, [C.c_void_p, _dp, C.c_int]),
    ("msmgb_copyin_simbox", C.c_int, [C.c_void_p, C.c_int, C.POINTER(Box), _ip, _ip, _dp, _dp]),
    ("msmgb_set_masses", C.c_int, [C.c_void_p, C.c_int, _dp]),
    ("msmgb_update_positions", C.c_int, [C.c_void_p, C.c_void_p]),
    ("msmgb_copyout_simbox", C.c_int, [C.c_void_p, _dp, _dp, _ip, _dp, C.c_int]),
    ("msmgb_copyout_force", C.c_int, [C.c_void_p, _dp, C.c_int]),
    ("msmgb_copyout_epot", C.c_int, [C.c_void_p, _dp, C.c_int]),
    ("msmgb_calekin", C.c_int, [C.c_void_p, _dp, C.c_int]),
    ("msmgb_copyout_den", C.c_int, [C.c_void_p, _dp, C.c_int]),
    ("msmgb_copyout_gid", C.c_int, [C.c_void_p, _ip]),
    ("msmgb_cal_neighborelist", C.c_int, [C.c_void_p]),
    ("msmgb_copyout_neighborelist", C.c_int, [C.c_void_p, _ip, _ip, C.c_int, C.c_int]),
    ("msmgb_predictor", C.c_int, [C.c_void_p, C.c_double]),
    ("msmgb_correction", C.c_int, [C.c_void_p, C.c_double]),
    ("msmgb_run_steps", C.c_int, [C.c_void_p, C.c_int, C.c_double, _ip]),
    ("msmgb_enqueue_steps", C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    ("msmgb_finish_steps", C.c_int, [C.c_void_p, C.c_double, _ip]),
    ("msmgb_time_steps", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_float), _ip]),
    ("msmgb_time_passes", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_float)]),
    ("msmgb_list_stats", C.c_int, [C.c_void_p, _ip, _dp]),
    ("msmgb_check_records", C.c_int, [C.c_void_p, _dp, _ip]),
    ("msmgb_tile_stats", C.c_int, [C.c_void_p, _ip, _ip, _dp, _ip]),
    ("msmgb_set_outer_skin", C.c_int, [C.c_void_p, C.c_double]),
    ("msmgb_set_boxshape", C.c_int, [C.c_void_p, C.c_int, _dp]),
    ("msmgb_rebuild_counts", C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("msmgb_time_rebuilds", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("msmgb_get_tuning", C.c_int, [C.c_void_p, _ip, C.POINTER(C.c_float)]),
    ("msmgb_set_tuning", C.c_int, [C.c_void_p, _ip]),
    ("msmgb_selftest_wait", C.c_int, [C.c_void_p]),
    ("msmgb_hvp", C.c_int, [C.c_void_p, _dp, _dp]),
    ("msmgb_time_hvp", C.c_int, [C.c_void_p, _dp, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    ("msmgb_param_adjoint", C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp]),
    ("msmgb_setfl_info", C.c_int, [C.c_char_p, _ip, _ip, _ip, _dp]),
    ("msmgb_setfl_tables", C.c_int, [C.c_char_p, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _dp, _dp]),
    ("msmgb_bonny_wheh_tables", C.c_int, [C.c_int, C.c_double, C.c_int, C.c_int, C.c_double,
                                          _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip, _dp]),
    ("msmgb_moldy_tables", C.c_int, [C.c_char_p, C.c_double, C.c_int, C.c_int, C.c_double,
                                     _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    ("msmgb_lspt_info", C.c_int, [C.c_char_p, C.c_int, _ip, _dp, _dp]),
    ("msmgb_lspt_tables", C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                    _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _dp]),
    ("msmgb_cr_param_tables", C.c_int, [_dp, C.c_double, C.c_int, _dp]),
    ("msmgb_calforce_noalloc", C.c_int, [C.POINTER(ForceNoAlloc)]),
    ("msmgb_create_forcetable", C.c_int, [C.c_int, _dp, C.c_double, C.c_int, C.c_int, C.c_double,
                                          _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    ("msmgb_import_info", C.c_int, [C.c_char_p, _ip, _ip, _ip, _ip, _ip, _ip, _ip]),
    ("msmgb_import_forcetable", C.c_int, [C.c_char_p, C.c_int, C.c_int, _ip, C.c_double, C.c_int, C.c_int,
                                          _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip, _ip, _dp, _ip]),
    ("msmgb_export_forcetable", C.c_int, [C.c_char_p, C.c_int, C.POINTER(ForceTable), _ip, _ip]),
    ("msmgb_set_steps_per_graph", C.c_int, [C.c_void_p, C.c_int]),
    ("msmgb_graph_launch_count", C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    ("msmgb_add_extforce", C.c_int, [C.c_void_p, C.c_char_p, EXTFORCE_FN, C.c_void_p]),
    ("msmgb_clear_extforce", C.c_int, [C.c_void_p]),
    ("msmgb_set_extforce_field", C.c_int, [C.c_void_p, C.c_void_p]),
]

_lib = None


def load(path: str = LIB_PATH):
    """Loads libmsmgb.so and declares every entry point; raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libmsmgb.so is not built (%s): run msmpscu_gb300.build.build() or "
                           "__graft_entry__.build(); there is no CPU fallback" % path)
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_names():
    return [s[0] for s in SIGNATURES]
