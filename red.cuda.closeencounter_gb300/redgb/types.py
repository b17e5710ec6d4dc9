"""Record layouts of the C ABI (include/redgb_types.h) as numpy dtypes and ctypes structs.

They are the reference's own records (red.cuda/red.type/red_type.h, gcc/Linux layout):
vec_t 32 B, param_t 32 B, body_metadata_t 24 B, orbelem_t 48 B, event_data_t 472 B.
"""
import ctypes

import numpy as np

VEC = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("w", "<f8")], align=True)
PARAM = np.dtype([("mass", "<f8"), ("radius", "<f8"), ("density", "<f8"), ("cd", "<f8")], align=True)
BODY_MD = np.dtype([("id", "<i4"), ("body_type", "<i4"), ("mig_type", "<i4"), ("mig_stop_at", "<f8")],
                   align=True)
ORBELEM = np.dtype([("sma", "<f8"), ("ecc", "<f8"), ("inc", "<f8"), ("peri", "<f8"), ("node", "<f8"),
                    ("mean", "<f8")], align=True)
EVENT = np.dtype([
    ("event_name", "<i4"), ("t", "<f8"), ("d", "<f8"),
    ("id1", "<i4"), ("idx1", "<i4"), ("p1", PARAM), ("r1", VEC), ("v1", VEC), ("oe1", ORBELEM),
    ("id2", "<i4"), ("idx2", "<i4"), ("p2", PARAM), ("r2", VEC), ("v2", VEC), ("oe2", ORBELEM),
    ("ps", PARAM), ("rs", VEC), ("vs", VEC), ("oes", ORBELEM)], align=True)

assert VEC.itemsize == 32 and PARAM.itemsize == 32 and BODY_MD.itemsize == 24
assert ORBELEM.itemsize == 48 and EVENT.itemsize == 472
assert EVENT.fields["r1"][1] == 64 and EVENT.fields["id2"][1] == 176 and EVENT.fields["oes"][1] == 424

# threshold_t (red_type.h:46-54)
THRESHOLD_HIT_CENTRUM_DISTANCE = 0
THRESHOLD_EJECTION_DISTANCE = 1
THRESHOLD_RADII_ENHANCE_FACTOR = 2
THRESHOLD_N = 5

# integrator_type_t (red_type.h:56-64)
INT_EULER, INT_RK2, INT_RK4, INT_RK5, INT_RKF78 = 0, 1, 2, 3, 4

# event_name_t (red_type.h:66-74)
EVENT_NONE, EVENT_HIT_CENTRUM, EVENT_EJECTION, EVENT_CLOSE_ENCOUNTER, EVENT_COLLISION = 0, 1, 2, 3, 4
EVENT_NAMES = ("NONE", "HIT_CENTRUM", "EJECTION", "CLOSE_ENCOUNTER", "COLLISION")

# body_type_t (red_type.h:90-99)
(BODY_STAR, BODY_GIANTPLANET, BODY_ROCKYPLANET, BODY_PROTOPLANET, BODY_SUPERPLANETESIMAL,
 BODY_PLANETESIMAL, BODY_TESTPARTICLE, BODY_PADDINGPARTICLE) = range(8)

GRAVITY_FP64, GRAVITY_MIXED = 0, 1
EVENT_TIME_CPU, EVENT_TIME_STAGE = 0, 1
FRAME_ASTRO, FRAME_BARY = 0, 1  # red_type.h:38-43 frame_center_t

# red.cuda/red.type/red_constants.h:21-22
GAUSS = 1.720209895e-2
GAUSS2 = 2.959122082855911025e-4
YEAR = 365.25  # red_constants.h YearToDay

STATUS = {0: "RG_OK", -1: "RG_ERR_ARG", -2: "RG_ERR_CUDA", -3: "RG_ERR_EVENT_OVERFLOW",
          -4: "RG_ERR_DT_NONFINITE", -5: "RG_ERR_STATE", -6: "RG_ERR_NOT_IMPLEMENTED",
          -7: "RG_ERR_NOMEM", -8: "RG_ERR_NO_DEVICE"}


class Counts(ctypes.Structure):
    """rg_counts_t: the number_of_bodies constructor arguments (number_of_bodies.h:7)."""
    _fields_ = [(n, ctypes.c_int32) for n in ("n_s", "n_gp", "n_rp", "n_pp", "n_spl", "n_pl", "n_tp")]

    def as_tuple(self):
        return tuple(getattr(self, f) for f, _ in self._fields_)

    @property
    def n_total(self):
        return sum(self.as_tuple())

    @property
    def n_si(self):
        return self.n_s + self.n_gp + self.n_rp + self.n_pp

    @property
    def n_massive(self):
        return self.n_si + self.n_spl + self.n_pl


class Counters(ctypes.Structure):
    """rg_counters_t."""
    _fields_ = [("n_failed_step", ctypes.c_int64), ("n_passed_step", ctypes.c_int64),
                ("n_tried_step", ctypes.c_int64),
                ("n_hit_centrum", ctypes.c_int64 * 3), ("n_ejection", ctypes.c_int64 * 3),
                ("n_collision", ctypes.c_int64 * 3), ("n_close_encounter", ctypes.c_int64 * 3),
                ("n_event", ctypes.c_int64 * 3), ("n_gravity_evals", ctypes.c_int64),
                ("n_pairs", ctypes.c_int64), ("n_kernels", ctypes.c_int64)]

    def as_dict(self):
        out = {}
        for f, _ in self._fields_:
            val = getattr(self, f)
            out[f] = list(val) if not isinstance(val, int) else val
        return out


class Profile(ctypes.Structure):
    """rg_profile_t: summed device time of timed launches."""
    _fields_ = [("gravity_launches", ctypes.c_int64), ("gravity_ms", ctypes.c_double),
                ("stage_launches", ctypes.c_int64), ("stage_ms", ctypes.c_double),
                ("other_launches", ctypes.c_int64), ("other_ms", ctypes.c_double)]


class Tune(ctypes.Structure):
    """rg_tune_t: the launch shape rg_autotune chose."""
    _fields_ = [("pairpar_sinks", ctypes.c_int32), ("rowseq_max_src", ctypes.c_int32),
                ("mixed_chunks", ctypes.c_int32), ("candidates", ctypes.c_int32),
                ("ms_per_eval", ctypes.c_double), ("ms_before", ctypes.c_double)]


STEP_REC = np.dtype([("sys", "<i4"), ("accepted", "<i4"), ("proposed", "<i4"), ("step", "<i4"), ("dt", "<f8"),
                     ("err", "<f8"), ("feat", "<f4", 8)], align=True)
assert STEP_REC.itemsize == 64

SYS_RUNNING, SYS_HELD, SYS_DONE, SYS_ERROR = 0, 1, 2, 3


class EnsStats(ctypes.Structure):
    """rg_ens_stats_t."""
    _fields_ = [("t_day", ctypes.c_double), ("dt_try_day", ctypes.c_double), ("dt_did_day", ctypes.c_double),
                ("n_tried_step", ctypes.c_int64), ("n_passed_step", ctypes.c_int64), ("n_failed_step", ctypes.c_int64),
                ("status", ctypes.c_int32), ("n_total", ctypes.c_int32), ("n_proposed", ctypes.c_int64),
                ("n_proposal_accepted", ctypes.c_int64), ("n_fallback", ctypes.c_int64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


def ptr(a):
    """ctypes void pointer to a contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


def event_key(e):
    """Comparison key of an event record: type, pair, step-independent fields."""
    return (int(e["event_name"]), int(e["id1"]), int(e["id2"]), int(e["idx1"]), int(e["idx2"]))
