"""ctypes mirrors of the POD structs in include/vec.h and the run presets.

The parameter set is the reference's INPUT file (src/initial.F90:142-172,
after the Ra/Q -> ck/F conversion of src/initial.F90:174-201) plus the
control flags hard-coded in src/main.F90:108-116 and the extensions
(eta(z) contrast, noise amplitude, precision form).
"""
import ctypes as C
import math

VEC_PREC_FP64 = 0
VEC_PREC_SPLIT = 1

# status codes of include/vec.h
STATUS = {
    0: "ok", -1: "bad nx", -2: "bad ny", -4: "nz < 6", -5: "allocation failed",
    -7: "unknown derivative flag", -8: "bad INPUT file", -12: "div B check failed",
    -20: "non-finite state", -30: "CUDA error", -31: "bad argument", -32: "unsupported size",
}

# field ids (include/vec.h enum vec_field)
F_R, F_T, F_U, F_V, F_W, F_BX, F_BY, F_BZ, F_JSQ, F_POL, F_TOR = range(11)
F_RDOT, F_TDOT, F_UDOT, F_VDOT, F_WDOT, F_POLDOT, F_TORDOT = 16, 19, 22, 25, 28, 31, 34
FIELD_NAMES = {"r": F_R, "t": F_T, "u": F_U, "v": F_V, "w": F_W, "bx": F_BX, "by": F_BY,
               "bz": F_BZ, "jsq": F_JSQ, "pol": F_POL, "tor": F_TOR}
for _n, _b in (("rdot", F_RDOT), ("tdot", F_TDOT), ("udot", F_UDOT), ("vdot", F_VDOT),
               ("wdot", F_WDOT), ("poldot", F_POLDOT), ("tordot", F_TORDOT)):
    for _s in range(3):
        FIELD_NAMES[f"{_n}{_s + 1}"] = _b + _s
M_BXBAR, M_BYBAR, M_BXBARDOT, M_BYBARDOT = 0, 1, 2, 5
M_KAPPA, M_DKAPPA, M_ETA, M_DETA = 8, 9, 10, 11
MEAN_NAMES = {"bxbar": M_BXBAR, "bybar": M_BYBAR, "kappa": M_KAPPA, "dkappa": M_DKAPPA,
              "eta": M_ETA, "deta": M_DETA}
for _s in range(3):
    MEAN_NAMES[f"bxbardot{_s + 1}"] = M_BXBARDOT + _s
    MEAN_NAMES[f"bybardot{_s + 1}"] = M_BYBARDOT + _s

STATE_FIELDS = ("r", "t", "u", "v", "w", "bx", "by", "bz", "jsq", "pol", "tor")


class VecParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "gamma", "sigma", "theta", "ck", "cm", "f", "tayl", "psi", "zeta", "xmax",
        "ymax", "sf", "rayl", "chand", "eta_contrast", "noise_amp")] + \
        [(n, C.c_int32) for n in (
            "nx", "ny", "nz", "nframe", "ntotal", "ndu06", "ndu16", "ndurestart",
            "dalias", "kinematic", "radbc", "constflux", "perfect", "dynamo",
            "kappa_uniform", "seed_base", "precision", "diag_cadence")]

    def copy(self):
        p = VecParams()
        C.pointer(p)[0] = self
        return p

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class VecScalars(C.Structure):
    _fields_ = [("dt", C.c_double), ("dt1", C.c_double), ("dt2", C.c_double),
                ("ttime", C.c_double), ("iter", C.c_int32), ("nit", C.c_int32),
                ("first", C.c_int32), ("second", C.c_int32)]


DIAG_FIELDS = ("ubar", "vbar", "kenergy", "menergy", "nusselt", "divbmax", "divbmin",
               "rmin", "rmax", "tmin", "tmax", "umin", "umax", "vmin", "vmax", "wmin",
               "wmax", "bxmin", "bxmax", "bymin", "bymax", "bzmin", "bzmax", "machmin",
               "machmax", "alfvenmin", "alfvenmax", "rmsmin", "rmsmax")


class VecDiag(C.Structure):
    _fields_ = [(n, C.c_double) for n in DIAG_FIELDS]

    def as_dict(self):
        return {n: getattr(self, n) for n in DIAG_FIELDS}


def ck_from_rayleigh(ra, theta, cm, sigma, gamma):
    """ck for flag=2 (Ra given), src/initial.F90:186-198."""
    return math.sqrt((((cm + 1.0) * theta * theta) / (sigma * ra * gamma))
                     * (cm + 1.0 - (cm * gamma))
                     * (1.0 + (0.5 * theta)) ** ((2.0 * cm) - 1.0))


def default_params():
    """bin/INPUT values with the control flags of src/main.F90:108-116."""
    p = VecParams()
    p.gamma, p.sigma, p.theta, p.cm = 1.4, 1.0, 10.0, 1.0
    p.tayl, p.psi, p.zeta, p.xmax, p.ymax, p.sf = 0.0, 1.570796327, 0.2, 4.0, 4.0, 0.2
    p.rayl, p.chand = 1.0e5, 2500.0
    p.ck = ck_from_rayleigh(p.rayl, p.theta, p.cm, p.sigma, p.gamma)
    p.f = p.chand * (p.zeta * p.sigma * p.ck * p.ck)
    p.nx, p.ny, p.nz = 30, 30, 60
    p.nframe, p.ntotal, p.ndu06, p.ndu16, p.ndurestart = 0, 50000, 5000, 10000, 10000
    p.dalias, p.kinematic, p.radbc, p.constflux, p.perfect, p.dynamo = 1, 0, 0, 0, 0, 0
    p.eta_contrast, p.noise_amp, p.kappa_uniform, p.seed_base = 1.0, 0.1, 0, 1996
    p.precision, p.diag_cadence = VEC_PREC_FP64, 1
    return p


def convection_params(nx, ny, nz, ra=1.0e5, q=100.0, theta=9.0, eta_contrast=5.0,
                      noise=1.0e-3, sf=0.3, precision=VEC_PREC_FP64, aspect=4.0):
    """Polytropic m=1 layer, density contrast (1+theta)^m, Pr=1, gamma=1.4,
    zeta=0.2, fixed-T top / fixed-flux bottom, vertical seed field Bz=1,
    eta(z) = eta0 (1 + (contrast-1) z), seeded uniform +-noise on T."""
    p = default_params()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.xmax = p.ymax = aspect
    p.theta, p.cm, p.sigma, p.gamma, p.zeta = theta, 1.0, 1.0, 1.4, 0.2
    p.rayl, p.chand = ra, q
    p.ck = ck_from_rayleigh(ra, theta, p.cm, p.sigma, p.gamma)
    p.f = q * (p.zeta * p.sigma * p.ck * p.ck)
    p.constflux, p.perfect = 1, 0
    p.eta_contrast, p.noise_amp, p.sf = eta_contrast, noise, sf
    p.precision = precision
    p.ntotal, p.ndu06, p.ndu16 = 1000, 1000, 1000000
    return p


# The workloads: the CPU-runnable reference case and the 256^2 x 129 GB300 case.
def config0(**kw):
    """64x64x65, Ra 1e5, Q 100, eta contrast 5, 1000 AB3 steps at CFL 0.3."""
    return convection_params(64, 64, 65, eta_contrast=5.0, **kw)


def config1(**kw):
    """256x256x129, Ra 1e5, Q 100, eta contrast 20."""
    return convection_params(256, 256, 129, eta_contrast=20.0, **kw)


def config4(**kw):
    """1024x1024x513, Ra 1e7, Q 1e4, eta contrast 50, theta 19 (density
    contrast 20), +-1e-4 temperature noise."""
    return convection_params(1024, 1024, 513, ra=1.0e7, q=1.0e4, theta=19.0, eta_contrast=50.0,
                             noise=1.0e-4, **kw)


def config2_members(seed=20240, precision=VEC_PREC_SPLIT):
    """The 48-member ensemble: 16 each at 64^2 x 65, 128^2 x 97 and
    192^2 x 129; Ra log-uniform in [1e4, 1e6], Q in {0, 100, 1000}, eta
    contrast in {1, 5, 20}, drawn from a seeded generator; m=1, density
    contrast 10; seeded +-1e-3 temperature noise (a distinct noise seed per
    member)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for g, (n, nz) in enumerate(((64, 65), (128, 97), (192, 129))):
        for i in range(16):
            ra = float(10.0 ** rng.uniform(4.0, 6.0))
            q = float(rng.choice([0.0, 100.0, 1000.0]))
            eta = float(rng.choice([1.0, 5.0, 20.0]))
            p = convection_params(n, n, nz, ra=ra, q=q, eta_contrast=eta, precision=precision)
            p.seed_base = 1996 + 7919 * (16 * g + i)
            p.ntotal, p.ndu06 = 5000, 1000000
            out.append(p)
    return out


class VecClosureReport(C.Structure):
    """include/vec.h vec_closure_report."""
    _fields_ = [("judges", C.c_int32), ("pad_", C.c_int32), ("coarse_steps", C.c_int64),
                ("fine_steps", C.c_int64), ("fallback_step", C.c_int64), ("last_err", C.c_double * 3),
                ("max_err", C.c_double * 3), ("end_time", C.c_double), ("nseries", C.c_int32),
                ("divb_fail", C.c_int32), ("blowup", C.c_int32), ("pad2_", C.c_int32)]


class VecSnapshot(C.Structure):
    """include/vec.h vec_snapshot (fields: R, T, U, V, W, Bx, By, Bz)."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("iteration", C.c_int32),
                ("version", C.c_int32), ("pad_", C.c_int32), ("time", C.c_double), ("timestep", C.c_double)] + \
               [(n, C.c_double) for n in ("gamma", "sigma", "theta", "ck", "cm", "f", "tayl", "psi", "zeta",
                                          "xmax", "ymax")] + \
               [("history", C.c_char * 80), ("fields", C.c_void_p * 8)]
