"""ctypes loader for the FP64 CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY.  The test suite, the smoke check and the
CPU-baseline leg of ``bench.py`` import this module as the reference answer; the
product (the CUDA library and the ``annmap`` package) never does.

The oracle restates the reference's CPU map path; see oracle.h for the file
and line of the reference each function follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_LOCK = threading.Lock()


class OrcHpx(C.Structure):
    _fields_ = [("nside", C.c_int64), ("npix", C.c_int64), ("ncap", C.c_int64),
                ("fact1", C.c_double), ("fact2", C.c_double)]


class OrcParams(C.Structure):
    _fields_ = [
        ("h100", C.c_double), ("Omega_M", C.c_double), ("Lbox_in_Mpc", C.c_double),
        ("mass_to_Msun", C.c_double), ("redshift", C.c_double),
        ("centerpos", C.c_double * 3), ("obs_pos", C.c_double * 3),
        ("align_vec", C.c_double * 3), ("particle_masses", C.c_double * 10),
        ("nside", C.c_int),
        ("rho_crit_in_cgs", C.c_double), ("length_to_cgs", C.c_double),
        ("mass_to_cgs", C.c_double), ("density_to_cgs", C.c_double),
        ("time_to_cgs", C.c_double), ("velocity_to_cgs", C.c_double),
        ("annihilation_flux_to_cgs", C.c_double),
        ("otheta", C.c_double), ("ophi", C.c_double),
        ("rotmatrix", (C.c_double * 3) * 3),
        ("unit_factor", C.c_double), ("hires_threshold", C.c_double),
        ("npix", C.c_int64), ("dOmega", C.c_double), ("theta0", C.c_double),
        ("flux_model", C.c_int), ("decay_unit_factor", C.c_double),
        ("halo_x", C.POINTER(C.c_float)), ("halo_y", C.POINTER(C.c_float)),
        ("halo_z", C.POINTER(C.c_float)), ("halo_r", C.POINTER(C.c_float)), ("n_halos", C.c_int),
        ("exact_boost", C.c_int),
    ]


class OrcStats(C.Structure):
    _fields_ = [("kept", C.c_int64), ("skipped", C.c_int64),
                ("single_small", C.c_int64), ("single_disc", C.c_int64),
                ("disc", C.c_int64), ("deposits", C.c_int64)]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, seconds)."""
    so = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("healpix_ring.c", "annmap_oracle.c", "oracle.h")]
    stale = (not os.path.exists(so)) or any(os.path.getmtime(s) > os.path.getmtime(so) for s in srcs)
    if force or stale:
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return so


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            L = C.CDLL(build())
            P = C.POINTER
            f32 = P(C.c_float)
            L.orc_hpx_init.argtypes = [P(OrcHpx), C.c_int64]
            L.orc_hpx_ang2pix.argtypes = [P(OrcHpx), C.c_double, C.c_double]
            L.orc_hpx_ang2pix.restype = C.c_int64
            L.orc_hpx_pix2vec.argtypes = [P(OrcHpx), C.c_int64, P(C.c_double)]
            L.orc_hpx_pix2ang.argtypes = [P(OrcHpx), C.c_int64, P(C.c_double), P(C.c_double)]
            L.orc_hpx_ring_above.argtypes = [P(OrcHpx), C.c_double]
            L.orc_hpx_ring_above.restype = C.c_int64
            L.orc_hpx_ring2z.argtypes = [P(OrcHpx), C.c_int64]
            L.orc_hpx_ring2z.restype = C.c_double
            L.orc_hpx_ring_info.argtypes = [P(OrcHpx), C.c_int64, P(C.c_int64), P(C.c_int64), P(C.c_int)]
            L.orc_hpx_query_disc.argtypes = [P(OrcHpx), C.c_double, C.c_double, C.c_double,
                                             P(C.c_int64), P(C.c_int64)]
            L.orc_hpx_query_disc.restype = C.c_int64
            L.orc_hpx_query_disc_list.argtypes = [P(OrcHpx), C.c_double, C.c_double, C.c_double,
                                                  P(C.c_int32)]
            L.orc_hpx_query_disc_list.restype = C.c_int64
            L.orc_params_setup.argtypes = [P(OrcParams)]
            L.orc_render.argtypes = [P(OrcParams), f32, f32, f32, f32, f32, f32, C.c_int64,
                                     P(C.c_double), P(OrcStats), C.c_int]
            L.orc_render.restype = C.c_int
            L.orc_render_v.argtypes = [P(OrcParams), f32, f32, f32, f32, f32, f32, f32, C.c_int64,
                                       P(C.c_double), P(OrcStats), C.c_int]
            L.orc_render_v.restype = C.c_int
            L.orc_finalize.argtypes = [P(OrcParams), P(C.c_double)]
            L.orc_finalize.restype = C.c_double
            L.orc_particle_geom.argtypes = [P(OrcParams), C.c_float, C.c_float, C.c_float,
                                            C.c_float, C.c_float, C.c_float, P(C.c_double)]
            L.orc_particle_loss.argtypes = [P(OrcParams)] + [C.c_double] * 6 + [
                P(C.c_double), P(C.c_uint64)]
            L.orc_particle_loss.restype = C.c_double
            d64 = P(C.c_double)
            L.orc_particle_losses.argtypes = [P(OrcParams), d64, d64, d64, d64, d64, d64,
                                              C.c_int64, d64, d64, P(C.c_uint64)]
            L.orc_adjoint.argtypes = [P(OrcParams), f32, f32, f32, f32, f32, f32, C.c_int64,
                                      P(C.c_double), P(C.c_double), P(C.c_double)]
            L.orc_adjoint.restype = C.c_int
            L.orc_particle_losses_v.argtypes = [P(OrcParams), d64, d64, d64, d64, d64, d64, d64,
                                                C.c_int64, d64, d64, P(C.c_uint64)]
            L.orc_adjoint_v.argtypes = [P(OrcParams), f32, f32, f32, f32, f32, f32, f32, C.c_int64,
                                        P(C.c_double), P(C.c_double), P(C.c_double)]
            L.orc_adjoint_v.restype = C.c_int
            _LIB = L
    return _LIB


# ---------------------------------------------------------------- HEALPix
class Healpix:
    """RING-scheme HEALPix functions of the oracle (FP64)."""

    def __init__(self, nside: int):
        self.b = OrcHpx()
        lib().orc_hpx_init(C.byref(self.b), nside)
        self.nside, self.npix = nside, 12 * nside * nside

    def ang2pix(self, theta, phi):
        return lib().orc_hpx_ang2pix(C.byref(self.b), float(theta), float(phi))

    def pix2vec(self, pix):
        v = (C.c_double * 3)()
        lib().orc_hpx_pix2vec(C.byref(self.b), int(pix), v)
        return np.array(v[:])

    def pix2ang(self, pix):
        t, p = C.c_double(), C.c_double()
        lib().orc_hpx_pix2ang(C.byref(self.b), int(pix), C.byref(t), C.byref(p))
        return t.value, p.value

    def ring_above(self, z):
        return lib().orc_hpx_ring_above(C.byref(self.b), float(z))

    def ring2z(self, ring):
        return lib().orc_hpx_ring2z(C.byref(self.b), int(ring))

    def ring_info(self, ring):
        s, n, sh = C.c_int64(), C.c_int64(), C.c_int()
        lib().orc_hpx_ring_info(C.byref(self.b), int(ring), C.byref(s), C.byref(n), C.byref(sh))
        return s.value, n.value, bool(sh.value)

    def query_disc(self, theta, phi, radius) -> np.ndarray:
        tot = C.c_int64()
        lib().orc_hpx_query_disc(C.byref(self.b), float(theta), float(phi), float(radius), None,
                                 C.byref(tot))
        out = np.empty(max(tot.value, 1), dtype=np.int32)
        n = lib().orc_hpx_query_disc_list(C.byref(self.b), float(theta), float(phi), float(radius),
                                          out.ctypes.data_as(C.POINTER(C.c_int32)))
        return out[:n]


# ---------------------------------------------------------------- params
def make_params(*, nside, obs_pos, centerpos, align_vec, h100=0.73, Omega_M=0.238,
                Lbox_in_Mpc=0.001, mass_to_Msun=1.0, particle_masses=(0.0,),
                redshift=0.0, flux_model=0, halos=None, exact_boost=False) -> OrcParams:
    """halos: optional (x, y, z, radius) arrays of the ann_core_nosom law's
    halo table (kept alive on the returned object).  exact_boost: the halo-
    core factor on unrounded positions (for central differences; the
    reference rounds them to float)."""
    p = OrcParams()
    p.flux_model = int(flux_model)
    p.exact_boost = int(bool(exact_boost))
    if halos is not None:
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in halos]
        p._halos = arrs
        p.halo_x, p.halo_y, p.halo_z, p.halo_r = [a.ctypes.data_as(C.POINTER(C.c_float)) for a in arrs]
        p.n_halos = len(arrs[0])
    p.h100, p.Omega_M, p.Lbox_in_Mpc, p.mass_to_Msun, p.redshift = (
        h100, Omega_M, Lbox_in_Mpc, mass_to_Msun, redshift)
    for i in range(3):
        p.centerpos[i], p.obs_pos[i], p.align_vec[i] = centerpos[i], obs_pos[i], align_vec[i]
    for i in range(10):
        p.particle_masses[i] = particle_masses[i] if i < len(particle_masses) else 0.0
    p.nside = int(nside)
    lib().orc_params_setup(C.byref(p))
    return p


def rotmatrix(p: OrcParams) -> np.ndarray:
    return np.array([[p.rotmatrix[i][j] for j in range(3)] for i in range(3)])


# ---------------------------------------------------------------- map
def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


def render(p: OrcParams, parts: dict, nthreads: int = 1, finalize: bool = True):
    """Runs the restated CPU map loop.  ``parts`` holds float32 arrays
    x, y, z, m, rho, h.  Returns (map, stats, totalC)."""
    keep = []
    ptrs = []
    for k in ("m", "rho", "h", "x", "y", "z"):
        a, ptr = _f32(parts[k])
        keep.append(a)
        ptrs.append(ptr)
    n = len(keep[0])
    sv = None
    if parts.get("sigmav") is not None:
        sva, sv = _f32(parts["sigmav"])
        keep.append(sva)
    mp = np.zeros(int(p.npix), dtype=np.float64)
    st = OrcStats()
    rc = lib().orc_render_v(C.byref(p), *ptrs, sv, n, mp.ctypes.data_as(C.POINTER(C.c_double)),
                            C.byref(st), int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle render failed")
    total = None
    if finalize:
        total = lib().orc_finalize(C.byref(p), mp.ctypes.data_as(C.POINTER(C.c_double)))
    stats = {k: getattr(st, k) for k, _ in OrcStats._fields_}
    return mp, stats, total


def particle_geom(p: OrcParams, m, rho, h, x, y, z) -> dict:
    out = (C.c_double * 8)()
    lib().orc_particle_geom(C.byref(p), m, rho, h, x, y, z, out)
    keys = ("d", "flux", "costheta", "phi", "theta", "ar", "pix", "kept")
    return dict(zip(keys, out[:]))


# ---------------------------------------------------------------- adjoint
def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def adjoint(p: OrcParams, parts: dict, G) -> tuple:
    """FP64 CPU reference adjoint of L = sum_p G[p] map[p] (map after the
    dOmega division).  Returns (grad [6, n] for x, y, z, m, rho, h,
    oacc[12] = (sum_i dL/du_i, dL/drot row-major))."""
    keep, ptrs = [], []
    for k in ("m", "rho", "h", "x", "y", "z"):
        a, ptr = _f32(parts[k])
        keep.append(a)
        ptrs.append(ptr)
    n = len(keep[0])
    G = np.ascontiguousarray(G, dtype=np.float64)
    grad = np.zeros((6, n), dtype=np.float64)
    oacc = np.zeros(12, dtype=np.float64)
    if parts.get("sigmav") is not None:     # the somv, somv2 and pwave laws
        sv, svp = _f32(parts["sigmav"])
        rc = lib().orc_adjoint_v(C.byref(p), *ptrs, svp, n, _dptr(G), _dptr(grad), _dptr(oacc))
    else:
        rc = lib().orc_adjoint(C.byref(p), *ptrs, n, _dptr(G), _dptr(grad), _dptr(oacc))
    if rc != 0:
        raise RuntimeError("oracle adjoint failed")
    return grad, oacc


def particle_loss(p: OrcParams, m, rho, h, x, y, z, G) -> tuple:
    """(L_i, pixel-set signature) of one particle from double inputs."""
    sig = C.c_uint64()
    L = lib().orc_particle_loss(C.byref(p), float(m), float(rho), float(h), float(x), float(y),
                                float(z), _dptr(G), C.byref(sig))
    return L, sig.value


def particle_losses(p: OrcParams, parts: dict, G) -> tuple:
    """(L_i, signature_i) of every particle; ``parts`` may hold float64
    arrays (unrounded inputs for finite differences)."""
    arrs = [np.ascontiguousarray(parts[k], dtype=np.float64) for k in ("m", "rho", "h", "x", "y", "z")]
    n = len(arrs[0])
    G = np.ascontiguousarray(G, dtype=np.float64)
    L = np.zeros(n)
    sig = np.zeros(n, dtype=np.uint64)
    sigp = sig.ctypes.data_as(C.POINTER(C.c_uint64))
    if parts.get("sigmav") is not None:     # the somv, somv2 and pwave laws
        sv = np.ascontiguousarray(parts["sigmav"], dtype=np.float64)
        lib().orc_particle_losses_v(C.byref(p), *[_dptr(a) for a in arrs], _dptr(sv), n, _dptr(G),
                                    _dptr(L), sigp)
    else:
        lib().orc_particle_losses(C.byref(p), *[_dptr(a) for a in arrs], n, _dptr(G), _dptr(L),
                                  sigp)
    return L, sig


def with_observer(p: OrcParams, obs_pos) -> OrcParams:
    """A copy of p with another observer position (all derived fields redone)."""
    q = OrcParams()
    C.memmove(C.byref(q), C.byref(p), C.sizeof(OrcParams))
    if hasattr(p, "_halos"):
        q._halos = p._halos
    for i in range(3):
        q.obs_pos[i] = float(obs_pos[i])
    lib().orc_params_setup(C.byref(q))
    return q


def rotation_jacobian_fd(p: OrcParams, rel_step: float = 1e-4) -> np.ndarray:
    """d rotmatrix / d obs_pos by central differences of the parameter set-up
    with one Richardson step: jac[e, k] for the row-major element e."""
    o = np.array(p.obs_pos[:], dtype=np.float64)
    radius = np.linalg.norm(o - np.array(p.centerpos[:]))
    jac = np.zeros((9, 3))
    for k in range(3):
        def D(step):
            op, om = o.copy(), o.copy()
            op[k] += step
            om[k] -= step
            return (rotmatrix(with_observer(p, op)) - rotmatrix(with_observer(p, om))).reshape(9) / (2 * step)
        hstep = rel_step * radius
        jac[:, k] = (4.0 * D(hstep / 2) - D(hstep)) / 3.0
    return jac


def observer_grad(p: OrcParams, oacc, jac=None) -> np.ndarray:
    """dL/d(observer position) from the adjoint's sums: -sum_i dL/du_i plus
    the rotation's dependence on the observer."""
    if jac is None:
        jac = rotation_jacobian_fd(p)
    return -np.asarray(oacc[:3]) + np.asarray(oacc[3:]) @ jac
