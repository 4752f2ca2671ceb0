"""Parameters: the reference's info-file configuration, mirrored.

Follows src/parameters.h:4-57 and src/parameters.cpp:291-483 -- the same
keys, the same tokenisation (a line is split on single spaces; the first
token is the key, the second (``=``) is skipped, values start at the third;
lines whose first token starts with ``#`` are comments), the same defaults
(Nside 512, 10^7 buffered particles, ``test = -1``, native data) and the same
derived fields.  The unit set-up and the observer rotation are computed by
the native library (dmann_code_units / dmann_observer_rotation, restating
Parameters::setupUnits / setupParams / setupRotation) so the Python, C++ and
CUDA paths share one implementation.

Differences from the reference, where it would crash or read garbage: a key
without a value raises ``ValueError``; a missing required key raises
``ValueError`` when the derived fields are computed; ``obs_pos`` equal to
``centerpos`` raises (the reference's angles are NaN).  ``set_observer`` and
``set_nside`` are programmatic setters the reference lacks (its observer is
private); batched rendering needs them.
"""
from __future__ import annotations

import ctypes as C
import math
import re
from dataclasses import dataclass, field

from . import _lib

MAX_NUM_MASS_RES = 10
_NUM = re.compile(r"^\s*[+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan)", re.I)
_INT = re.compile(r"^\s*[+-]?\d+")


def atof(s: str) -> float:
    """C atof: the longest numeric prefix, 0.0 when there is none."""
    m = _NUM.match(s)
    return float(m.group(0)) if m else 0.0


def atoi(s: str) -> int:
    m = _INT.match(s)
    return int(m.group(0)) if m else 0


@dataclass
class MapInfo:
    """src/datatypes.h:236-254 (Map::setNside)."""
    Nside: int = 512
    Npix: int = 12 * 512 * 512
    dOmega: float = 4 * math.pi / (12 * 512 * 512)
    theta0: float = 0.0
    projection: str = ""

    def setNside(self, nside: int):
        self.Nside = int(nside)
        self.Npix = 12 * self.Nside * self.Nside
        self.dOmega = 4 * math.pi / self.Npix
        self.theta0 = 0.0


@dataclass
class CodeUnits:
    mass_to_cgs: float = 0.0
    mass_to_Msun: float = 0.0
    length_to_Mpc: float = 0.0
    length_to_cgs: float = 0.0
    time_to_cgs: float = 0.0
    velocity_to_cgs: float = 0.0
    density_to_cgs: float = 0.0
    annihilation_flux_to_cgs: float = 0.0


@dataclass
class Params:
    """src/datatypes.h:220-232."""
    z: float = 0.0
    cpos: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    cvel: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    opos: list = field(default_factory=lambda: [0.0, 0.0, 0.0])
    otheta: float = 0.0
    ophi: float = 0.0
    Lbox_in_Mpc: float = 0.0
    particle_numbers: list = field(default_factory=lambda: [0] * MAX_NUM_MASS_RES)
    particle_masses: list = field(default_factory=lambda: [0.0] * MAX_NUM_MASS_RES)
    particle_masses_in_Msun: list = field(default_factory=lambda: [0.0] * MAX_NUM_MASS_RES)


class Parameters:
    """Mirror of the reference's Parameters class (src/parameters.h:4-57)."""

    REQUIRED = ("h100", "Lbox_in_Mpc")

    def __init__(self, info_file: str | None = None, *, text: str | None = None):
        # Parameters::initialize (parameters.cpp:291-308) and constructor defaults
        self.map = MapInfo()
        self.map.setNside(512)
        self.memParts = 10000000
        self.testNum = -1
        self.isNative = True
        self.partFile = self.densFile = self.hsmFile = self.dspFile = ""
        self.nativeDatafile = ""
        self.outputFileName = ""
        self.maskFileName = ""
        self.isMask = False
        self.redshift = 0.0
        self.info = {"particle_masses": [0.0] * MAX_NUM_MASS_RES,
                     "particle_numbers": [0] * MAX_NUM_MASS_RES, "mass_to_Msun": -1.0,
                     "centerpos": [0.0, 0.0, 0.0], "centervel": [0.0, 0.0, 0.0]}
        self.halo = {}
        self.align_vector = None
        self.obs_pos = None
        self.codeunits = CodeUnits()
        self.params = Params()
        self.rotmatrix = [[1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]
        self.unit_factor = 1.0
        if info_file is not None or text is not None:
            if text is None:
                with open(info_file, "r") as f:
                    text = f.read()
            self._parse(text)
            self.setup()

    # ------------------------------------------------------------------ parse
    def _parse(self, text: str):
        info = self.info
        for raw in text.split("\n"):
            line = raw
            if len(line) == 0:
                continue
            toks = [t for t in line.split(" ") if t != ""]
            if not toks:
                continue
            key = toks[0]
            if key.startswith("#"):
                continue
            vals = toks[2:]

            def need(k=1):
                if len(vals) < k:
                    raise ValueError(f"info file: key {key!r} needs {k} value(s)")
                return vals

            if key in ("Omega_M", "h100", "n_s", "sigma_8", "Lbox_in_Mpc", "mass_to_Msun"):
                info[key] = atof(need()[0])
            elif key == "particle_masses":
                v = need()
                for i in range(min(len(v), MAX_NUM_MASS_RES)):
                    info["particle_masses"][i] = atof(v[i])
            elif key == "particle_numbers":
                v = need()
                for i in range(min(len(v), MAX_NUM_MASS_RES)):
                    info["particle_numbers"][i] = atoi(v[i])
            elif key in ("centerpos", "centervel"):
                info[key] = [atof(x) for x in need(3)[:3]]
            elif key in ("Mvir_in_Msun", "M200_in_Msun", "M200crit_in_Msun", "Rvir_in_Mpc",
                         "R200_in_Mpc", "R200crit_in_Mpc", "Vmax_in_kms", "RVmax_in_kpc",
                         "rconverg_in_kpc"):
                self.halo[key] = atof(need()[0])
            elif key in ("params_NFW", "params_GNFW", "params_Einasto"):
                self.halo[key] = [atof(x) for x in need(3)[:3]]
            elif key == "align_vec":
                self.align_vector = [atof(x) for x in need(3)[:3]]
            elif key == "obs_pos":
                self.obs_pos = [atof(x) for x in need(3)[:3]]
            elif key == "nside":
                self.map.setNside(atoi(need()[0]))
            elif key == "test":
                self.testNum = atoi(need()[0])
            elif key == "datafile":
                self.nativeDatafile = need()[0]
            elif key in ("partfile", "densfile", "hsmfile", "vdspfile"):
                attr = {"partfile": "partFile", "densfile": "densFile", "hsmfile": "hsmFile",
                        "vdspfile": "dspFile"}[key]
                setattr(self, attr, need()[0])
                self.isNative = False
            elif key == "outputmap":
                self.outputFileName = need()[0]
            elif key == "mem_buffer":
                self.memParts = atoi(need()[0])
            elif key == "mask":
                self.maskFileName = need()[0]
                self.isMask = True

    # ------------------------------------------------------------------ derive
    def setup(self):
        """setupUnits, setupOthers, setupHalo, setupParams, setupRotation."""
        for k in self.REQUIRED:
            if k not in self.info:
                raise ValueError(f"info file is missing {k!r}")
        if self.obs_pos is None or self.align_vector is None:
            raise ValueError("info file is missing obs_pos / align_vec")
        L = _lib.load()
        out = (C.c_double * 9)()
        L.dmann_code_units(self.info["h100"], self.info["Lbox_in_Mpc"], self.info["mass_to_Msun"], out)
        cu = self.codeunits
        (rho_crit, cu.length_to_cgs, cu.time_to_cgs, cu.density_to_cgs, cu.mass_to_cgs,
         cu.mass_to_Msun, cu.velocity_to_cgs, cu.annihilation_flux_to_cgs, self.unit_factor) = out[:]
        cu.length_to_Mpc = self.info["Lbox_in_Mpc"]
        self.rho_crit_in_cgs = rho_crit
        p = self.params
        p.z = self.redshift
        p.cpos = list(self.info["centerpos"])
        p.cvel = list(self.info["centervel"])
        p.opos = list(self.obs_pos)
        p.Lbox_in_Mpc = self.info["Lbox_in_Mpc"]
        j = 0
        p.particle_masses = [0.0] * MAX_NUM_MASS_RES
        p.particle_numbers = [0] * MAX_NUM_MASS_RES
        p.particle_masses_in_Msun = [0.0] * MAX_NUM_MASS_RES
        for i in range(MAX_NUM_MASS_RES):
            if self.info["particle_masses"][i] > 0:
                p.particle_numbers[j] = self.info["particle_numbers"][i]
                p.particle_masses[j] = self.info["particle_masses"][i]
                p.particle_masses_in_Msun[j] = (self.info["particle_masses"][i] * cu.mass_to_cgs /
                                                1.9889212e+33)
                j += 1
        self._rotation()

    def _rotation(self):
        L = _lib.load()
        d3 = lambda v: (C.c_double * 3)(*[float(x) for x in v])
        rot = (C.c_double * 9)()
        ang = (C.c_double * 2)()
        st = L.dmann_observer_rotation(d3(self.params.opos), d3(self.params.cpos),
                                       d3(self.align_vector), rot, ang)
        if st != 0:
            raise ValueError("observer position equals the halo centre")
        self.rotmatrix = [list(rot[0:3]), list(rot[3:6]), list(rot[6:9])]
        self.params.otheta, self.params.ophi = ang[0], ang[1]

    # ------------------------------------------------------------------ setters
    def set_observer(self, opos, align=None):
        self.obs_pos = [float(x) for x in opos]
        self.params.opos = list(self.obs_pos)
        if align is not None:
            self.align_vector = [float(x) for x in align]
        self._rotation()

    def set_nside(self, nside: int):
        self.map.setNside(nside)

    # ------------------------------------------------------------------ derived
    def flux_unit_factor(self, flux_model=0) -> float:
        """The unit factor of a flux law (dmann_flux_unit_factor; a number
        or a name of _lib.FLUX_LAWS): the annihilation laws share
        unit_factor, the decay law has its own."""
        if isinstance(flux_model, str):
            flux_model = _lib.FLUX_LAWS[flux_model]
        if flux_model == 0:
            return self.unit_factor
        L = _lib.load()
        out = (C.c_double * 1)()
        if L.dmann_flux_unit_factor(int(flux_model), self.info["h100"], self.info["Lbox_in_Mpc"],
                                    self.info["mass_to_Msun"], out) != 0:
            raise ValueError("unknown flux law")
        return out[0]

    @property
    def hires_threshold(self) -> float:
        L = _lib.load()
        arr = (C.c_double * MAX_NUM_MASS_RES)(*self.params.particle_masses)
        return L.dmann_hires_threshold(arr, MAX_NUM_MASS_RES)

    def rot_flat(self):
        return [self.rotmatrix[i][j] for i in range(3) for j in range(3)]

    @classmethod
    def for_synthetic(cls, particles, nside: int, **kw) -> "Parameters":
        """Parameters for a synthetic set (code length 1 kpc, masses in Msun)."""
        lines = ["Omega_M = 0.238", "h100 = 0.73", "Lbox_in_Mpc = 0.001", "mass_to_Msun = 1",
                 f"particle_masses = {particles.particle_mass!r}",
                 "centerpos = " + " ".join(repr(float(v)) for v in particles.centerpos),
                 "align_vec = " + " ".join(repr(float(v)) for v in particles.align_vec),
                 "obs_pos = " + " ".join(repr(float(v)) for v in particles.obs_pos),
                 f"nside = {int(nside)}"]
        return cls(text="\n".join(lines) + "\n")
