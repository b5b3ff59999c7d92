"""Parameter files in the reference's ``.in`` format.

Restates the subset of ``src/dlbc/parameters.d`` the timestep path needs:

* ``key = value`` lines, ``[section]`` headers (the section is prefixed to
  the key with a dot), ``//`` comments (``parseParameterLine``,
  ``parameters.d:215-246``);
* command-line overrides ``--parameter section.key=value`` are applied after
  the files, with no section (``parseParametersFromCli``, ``parameters.d:184-196``);
* values as D's ``std.conv.to!T`` reads them: numbers, ``true``/``false``,
  enum member names, ``"quoted"`` strings and ``[ ... ]`` arrays (nested).

``LBParams.from_dict`` then applies the reference's defaults
(``@("param")`` declarations and ``checkArrayParameterLength``, which fills
a missing array with zeros, ``parameters.d:258-278``).
"""
from __future__ import annotations

import dataclasses
import re
from typing import Any, Dict, Iterable, List, Optional, Sequence


class ParameterError(ValueError):
    """Raised where the reference logs a fatal error and exits."""


def _tokenize_value(s: str) -> Any:
    s = s.strip()
    pos = 0

    def skip_ws():
        nonlocal pos
        while pos < len(s) and s[pos].isspace():
            pos += 1

    def parse_item():
        nonlocal pos
        skip_ws()
        if pos >= len(s):
            raise ParameterError(f"unexpected end of value {s!r}")
        ch = s[pos]
        if ch == "[":
            pos += 1
            out = []
            skip_ws()
            if pos < len(s) and s[pos] == "]":
                pos += 1
                return out
            while True:
                out.append(parse_item())
                skip_ws()
                if pos < len(s) and s[pos] == ",":
                    pos += 1
                    continue
                if pos < len(s) and s[pos] == "]":
                    pos += 1
                    return out
                raise ParameterError(f"malformed array value {s!r}")
        if ch == '"':
            end = s.index('"', pos + 1)
            v = s[pos + 1 : end]
            pos = end + 1
            return v
        m = re.compile(r"[^,\[\]]+").match(s, pos)
        if not m:
            raise ParameterError(f"malformed value {s!r}")
        pos = m.end()
        return _scalar(m.group(0).strip())

    v = parse_item()
    skip_ws()
    if pos != len(s):
        # a bare string that contains brackets or commas (e.g. file names)
        return _scalar(s)
    return v


def _scalar(tok: str) -> Any:
    low = tok.lower()
    if low in ("true", "false"):
        return low == "true"
    try:
        if re.fullmatch(r"[+-]?\d+", tok):
            return int(tok)
        return float(tok)
    except ValueError:
        return tok


def parse_lines(lines: Iterable[str], into: Optional[Dict[str, Any]] = None,
                section: str = "") -> Dict[str, Any]:
    """Parse parameter lines into ``{qualified.key: value}``."""
    out: Dict[str, Any] = {} if into is None else into
    cur = section
    for raw in lines:
        line = raw
        cpos = line.find("//")
        if cpos >= 0:
            line = line[:cpos]
        apos = line.find("=")
        if apos > 0:
            key = line[:apos].strip()
            val = line[apos + 1 :].strip()
            full = f"{cur}.{key}" if cur else key
            out[full] = _tokenize_value(val) if val else ""
        else:
            for m in re.finditer(r"\[(.*?)\]", line):
                cur = m.group(1)
    return out


def read_parameter_files(files: Sequence[str], cli: Sequence[str] = ()) -> Dict[str, Any]:
    """Files in order, then ``--parameter`` overrides (no section)."""
    d: Dict[str, Any] = {}
    for f in files:
        with open(f) as fh:
            parse_lines(fh.read().splitlines(), d)
    if cli:
        parse_lines(list(cli), d, section="")
    return d


EQ_FORMS = {"SecondOrder": 0, "ThirdOrder": 1, "BDist2": 2}
PSI_FORMS = {"Linear": 0, "Exponential": 1}
AXES = {"X": 0, "Y": 1, "Z": 2}
MASK_INITS = {"None": 0, "File": 1, "Plates": 2, "Tube": 3, "Box": 4, "Walls": 5}
FLUID_INITS = ["None", "File", "Const", "EqDist", "EqDistPerturb", "EqDistPerturbFrac",
               "ConstRandom", "EqDistRandom", "EqDistSphere", "EqDistSphereFrac",
               "EqDistCylinder", "EqDistCylinderFrac", "EqDistTwoSpheres",
               "EqDistTwoSpheresFrac", "EqDistLamellae", "EqDistLamellaeFrac"]


def _enum(val: Any, table: Dict[str, int], name: str) -> int:
    if isinstance(val, int) and not isinstance(val, bool):
        return val
    if val not in table:
        raise ParameterError(f"{name}: unknown value {val!r}")
    return table[val]


def _arr(d: Dict[str, Any], key: str, n: int, strict: bool = False, fill: Any = 0.0) -> List[Any]:
    """checkArrayParameterLength (parameters.d:258-278)."""
    v = d.get(key, [])
    if not isinstance(v, list):
        v = [v]
    if len(v) == 0 and n != 0:
        if strict:
            raise ParameterError(f"Array parameter {key} must have length {n}.")
        return [fill] * n
    if len(v) != n:
        raise ParameterError(f"Array parameter {key} must have length {n}.")
    return list(v)


@dataclasses.dataclass
class LBParams:
    """The timestep path's parameter subset, with the reference's defaults."""
    d: int = 3
    q: int = 19
    gn: List[int] = dataclasses.field(default_factory=lambda: [64, 64, 64])
    components: int = 1
    field_names: List[str] = dataclasses.field(default_factory=list)
    timesteps: int = 0
    tau: List[float] = dataclasses.field(default_factory=list)
    eq_form: int = 0
    shan_chen: bool = False
    gcc: List[List[float]] = dataclasses.field(default_factory=list)
    gwc: List[float] = dataclasses.field(default_factory=list)
    psi_form: int = 0
    global_acc: List[float] = dataclasses.field(default_factory=list)
    # init
    fluid_init: List[int] = dataclasses.field(default_factory=list)
    fluid_densities: List[List[float]] = dataclasses.field(default_factory=list)
    fluid_perturb: List[float] = dataclasses.field(default_factory=list)
    random_reseed: List[bool] = dataclasses.field(default_factory=list)
    random_seed: List[int] = dataclasses.field(default_factory=list)
    seed: int = 0
    shift_seed_by_rank: bool = True
    init_radius: float = 0.0
    init_offset: List[float] = dataclasses.field(default_factory=list)
    init_separation: List[float] = dataclasses.field(default_factory=list)
    init_axis: int = 0
    interface_thickness: float = 0.0
    lamellae_widths: List[float] = dataclasses.field(default_factory=list)
    fluid_files: List[str] = dataclasses.field(default_factory=list)
    mask_init: int = 0
    mask_file: str = ""
    mask_axis: int = 0
    wall_offset: int = 0
    wall_thickness: int = 1
    dimension_has_wall: List[List[bool]] = dataclasses.field(default_factory=list)
    nc: List[int] = dataclasses.field(default_factory=list)
    # io
    simulation_name: str = ""
    output_path: str = "."
    freqs: Dict[str, int] = dataclasses.field(default_factory=dict)
    cp_freq: int = 0
    cp_keep: int = 1
    cp_path: str = "."
    start_output: int = 0
    enable_io: bool = True
    raw: Dict[str, Any] = dataclasses.field(default_factory=dict)

    @classmethod
    def from_dict(cls, d: Dict[str, Any], dq: str = "d3q19") -> "LBParams":
        dq = dq.lower()
        if dq == "d3q19":
            dim, q = 3, 19
        elif dq == "d2q9":
            dim, q = 2, 9
        elif dq == "d1q3":
            dim, q = 1, 3
        elif dq == "d1q5":
            dim, q = 1, 5
        else:
            raise ParameterError(f"unsupported connectivity {dq}")
        p = cls(d=dim, q=q, raw=dict(d))
        p.gn = [int(x) for x in _arr(d, "lattice.gn", dim, strict=True)]
        p.components = int(d.get("lb.components", 1))
        C = p.components
        p.field_names = [str(x) for x in _arr(d, "lb.fieldNames", C, strict=True, fill="")]
        p.timesteps = int(d.get("lb.timesteps", 0))
        p.tau = [float(x) for x in _arr(d, "lb.tau", C, strict=p.timesteps > 0)]
        p.eq_form = _enum(d.get("lb.eqdist.eqDistForm", "SecondOrder"), EQ_FORMS, "eqDistForm")
        p.shan_chen = bool(d.get("lb.force.enableShanChen", False))
        p.psi_form = _enum(d.get("lb.force.psiForm", "Linear"), PSI_FORMS, "psiForm")
        p.global_acc = [float(x) for x in _arr(d, "lb.force.globalAcc", dim)]
        if p.shan_chen:
            g = _arr(d, "lb.force.gcc", C, strict=True)
            p.gcc = [[float(x) for x in _arr({"k": row}, "k", C, strict=True)] for row in g]
        else:
            p.gcc = [[0.0] * C for _ in range(C)]
        p.gwc = [float(x) for x in _arr(d, "lb.force.gwc", C)]
        fi = _arr(d, "lb.init.fluidInit", C, fill="None")
        p.fluid_init = [FLUID_INITS.index(x) if isinstance(x, str) else int(x) for x in fi]
        fd = _arr(d, "lb.init.fluidDensities", C, fill=[])
        p.fluid_densities = [[float(v) for v in (row if isinstance(row, list) else [row])] for row in fd]
        p.fluid_perturb = [float(x) for x in _arr(d, "lb.init.fluidPerturb", C)]
        p.random_reseed = [bool(x) for x in _arr(d, "lb.init.randomReseed", C, fill=False)]
        p.random_seed = [int(x) for x in _arr(d, "lb.init.randomSeed", C, fill=0)]
        p.seed = int(d.get("random.seed", 0))
        p.shift_seed_by_rank = bool(d.get("random.shiftSeedByRank", True))
        p.init_radius = float(d.get("lb.init.initRadius", 0.0))
        p.init_offset = [float(x) for x in _arr(d, "lb.init.initOffset", dim)]
        p.init_separation = [float(x) for x in _arr(d, "lb.init.initSeparation", dim)]
        p.init_axis = _enum(d.get("lb.init.initAxis", "X"), AXES, "initAxis")
        p.interface_thickness = float(d.get("lb.init.interfaceThickness", 0.0))
        p.lamellae_widths = [float(x) for x in d.get("lb.init.lamellaeWidths", [])]
        p.fluid_files = [str(x) for x in _arr(d, "lb.init.fluidFiles", C, fill="")]
        p.mask_file = str(d.get("lb.mask.maskFile", ""))
        p.mask_init = _enum(d.get("lb.mask.maskInit", "None"), MASK_INITS, "maskInit")
        p.mask_axis = _enum(d.get("lb.mask.initAxis", "X"), AXES, "mask.initAxis")
        p.wall_offset = int(d.get("lb.mask.wallOffset", 0))
        p.wall_thickness = int(d.get("lb.mask.wallThickness", 1))
        dhw = _arr(d, "lb.mask.dimensionHasWall", dim, fill=[False, False])
        p.dimension_has_wall = [[bool(x) for x in _arr({"k": r}, "k", 2, fill=False)] for r in dhw]
        p.nc = [int(x) for x in d.get("parallel.nc", [])] or [0] * dim
        p.simulation_name = str(d.get("io.simulationName", ""))
        p.output_path = str(d.get("io.outputPath", "."))
        p.start_output = int(d.get("io.startOutput", 0))
        p.enable_io = bool(d.get("io.enableIO", True))
        for k in ("population", "density", "colour", "velocity", "force", "mask"):
            p.freqs[k] = int(d.get(f"lb.io.{k}Freq", 0))
        p.cp_freq = int(d.get("io.checkpoint.cpFreq", 0))
        p.cp_keep = int(d.get("io.checkpoint.cpKeep", 1))
        p.cp_path = str(d.get("io.checkpoint.cpPath", "."))
        return p
