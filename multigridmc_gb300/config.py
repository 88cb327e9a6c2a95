"""Run configurations in the reference's libconfig format.

``load_run(parameters_file)`` reads a parameters file of the reference's
driver (the groups that src/auxilliary/parameters.cc reads: general, lattice,
smoother, multigrid, sampling, prior, constantcorrelationlengthmodel or
periodiccorrelationlengthmodel, measurements) and the measurement file it names (dim, n,
measurement_locations, mean, variance), and builds the linear operator, the
right hand side and the multigrid parameters of the sampling path, so that a
``driver_mgmc`` configuration runs unchanged on the GPU sampler.

The parser covers the libconfig subset these files use: groups
``name = { ... };``, scalar settings ``name = value;`` (integers, floats,
booleans, strings), arrays and lists ``[ ... ]`` / ``( ... )``, and ``//``,
``#`` and ``/* */`` comments.
"""
import os
import re
from dataclasses import dataclass, field

import numpy as np

_TOKEN = re.compile(r'\s*(?:(/\*.*?\*/)|(//[^\n]*|#[^\n]*)|("(?:[^"\\]|\\.)*")|([A-Za-z_][A-Za-z0-9_\-]*)|'
                    r'([-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?[Ll]?)|(0[xX][0-9a-fA-F]+)|([=:;,{}\[\]()]))', re.S)


def _tokens(text):
    pos, out = 0, []
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            if text[pos:].strip() == "":
                break
            raise ValueError(f"libconfig: cannot parse at offset {pos}: {text[pos:pos + 20]!r}")
        pos = m.end()
        comment1, comment2, string, name, number, hexnum, punct = m.groups()
        if comment1 or comment2:
            continue
        if string is not None:
            out.append(("str", bytes(string[1:-1], "utf-8").decode("unicode_escape")))
        elif name is not None:
            low = name.lower()
            out.append(("bool", low == "true") if low in ("true", "false") else ("name", name))
        elif number is not None:
            num = number.rstrip("Ll")
            out.append(("num", int(num) if re.fullmatch(r"[-+]?\d+", num) else float(num)))
        elif hexnum is not None:
            out.append(("num", int(hexnum, 16)))
        else:
            out.append(("p", punct))
    return out


def parse_libconfig(text):
    """Parse libconfig text into nested dicts / lists / scalars."""
    toks = _tokens(text)
    pos = 0

    def peek():
        return toks[pos] if pos < len(toks) else (None, None)

    def take(kind=None, value=None):
        nonlocal pos
        t = peek()
        if t[0] is None or (kind and t[0] != kind) or (value is not None and t[1] != value):
            raise ValueError(f"libconfig: expected {value or kind}, found {t[1]!r}")
        pos += 1
        return t

    def value():
        k, v = peek()
        if k == "p" and v == "{":
            take("p", "{")
            g = settings("}")
            take("p", "}")
            return g
        if k == "p" and v in "[(":
            close = "]" if v == "[" else ")"
            take("p", v)
            items = []
            while peek() != ("p", close):
                items.append(value())
                if peek() == ("p", ","):
                    take("p", ",")
            take("p", close)
            return items
        if k in ("str", "num", "bool"):
            take()
            return v
        raise ValueError(f"libconfig: unexpected {v!r}")

    def settings(end):
        out = {}
        while peek()[0] is not None and peek() != ("p", end):
            name = take("name")[1]
            sep = peek()
            if sep == ("p", "=") or sep == ("p", ":"):
                take()
            out[name] = value()
            if peek() in (("p", ";"), ("p", ",")):
                take()
        return out

    root = settings(None)
    if pos != len(toks):
        raise ValueError("libconfig: trailing tokens")
    return root


def _read(path):
    with open(path) as fh:
        return parse_libconfig(fh.read())


@dataclass
class RunConfig:
    """The sampling-path part of a driver configuration."""
    dim: int
    shape: tuple
    operator: str
    Lambda: float
    multigrid: dict
    smoother: dict
    sampling: dict
    measurements: dict = field(default_factory=dict)
    measurement_data: dict = field(default_factory=dict)
    correlation: str = "constant"  # or "periodic": Lambda_min, Lambda_max below
    pdemodel: str = "shiftedlaplace_fd"  # or "shiftedlaplace_fem"
    Lambda_min: float = 0.0
    Lambda_max: float = 0.0

    @property
    def kappa_sq(self):
        """kappa^2 = 1 / Lambda^2 (correlationlength_model.hh:52) of the
        constant correlation-length model."""
        if self.correlation != "constant":
            raise ValueError("kappa^2 varies in space for the periodic model")
        return 1.0 / self.Lambda ** 2

    def multigrid_parameters(self):
        from . import MultigridParameters
        mg = self.multigrid
        return MultigridParameters(nlevel=int(mg["nlevel"]), smoother=str(mg["smoother"]),
                                   coarse_solver=str(mg["coarse_solver"]), npresmooth=int(mg["npresmooth"]),
                                   npostsmooth=int(mg["npostsmooth"]), ncoarsesmooth=int(mg["ncoarsesmooth"]),
                                   omega=float(mg["omega"]), cycle=int(mg["cycle"]),
                                   coarse_scaling=float(mg["coarse_scaling"]))

    def linear_operator(self):
        """The prior (ShiftedLaplaceFDOperator or ShiftedLaplaceFEMOperator) or the posterior
        (MeasuredOperator) of the configuration (driver_mgmc.cc:120-160)."""
        from . import LinearOperator
        fem = self.pdemodel == "shiftedlaplace_fem"
        if self.correlation == "periodic":
            build = LinearOperator.shifted_laplace_fem_periodic if fem else LinearOperator.shifted_laplace_fd_periodic
            op = build(self.shape, self.Lambda_min, self.Lambda_max)
        else:
            op = (LinearOperator.shifted_laplace_fem if fem else LinearOperator.shifted_laplace_fd)(self.shape,
                                                                                                  self.kappa_sq)
        if self.operator == "prior":
            return op
        ms, md = self.measurements, self.measurement_data
        n = int(md["n"])
        loc = np.asarray(md["measurement_locations"], np.float64).reshape(n, self.dim)
        return op.with_measurements(loc, np.asarray(md["variance"], np.float64),
                                    variance_scaling=float(ms["variance_scaling"]), radius=float(ms["radius"]),
                                    measure_global=bool(ms["measure_global"]),
                                    variance_global=float(ms["variance_global"]))

    def rhs(self, op=None):
        """f = B Sigma^{-1} y with y the measured means (and the global mean
        when measured): the right hand side whose sample mean is the
        posterior mean (sampling_time.cc:19, 28); zero for the prior."""
        op = op or self.linear_operator()
        if self.operator == "prior" or op.m == 0:
            return np.zeros(op.n)
        y = list(np.asarray(self.measurement_data["mean"], np.float64))
        if bool(self.measurements.get("measure_global", False)):
            y.append(float(self.measurements["mean_global"]))
        y = np.asarray(y)
        f = np.zeros(op.n)
        for j in range(op.m):
            sl = slice(op.B_ptr[j], op.B_ptr[j + 1])
            f[op.B_idx[sl]] += op.B_val[sl] * (y[j] / op.Sigma[j])
        return f

    def sample_location(self):
        return [float(v) for v in self.measurements.get("sample_location", [0.5] * self.dim)]


def load_run(parameters_file, measurements_file=None):
    """RunConfig from a driver parameters file (parameters.cc:50-360) and
    the measurement file it names (resolved relative to the parameters
    file when it is not found as given)."""
    root = _read(parameters_file)
    g = root["general"]
    dim = int(g["dim"])
    lat = root["lattice"]
    shape = tuple(int(lat[k]) for k in ("nx", "ny", "nz")[:dim])
    operator = str(g["operator"])
    if operator not in ("prior", "posterior"):
        raise ValueError("operator has to be 'prior' or 'posterior'")
    prior = root.get("prior", {"pdemodel": "shiftedlaplace_fd", "correlationlengthmodel": "constant"})
    model = prior.get("correlationlengthmodel")
    if prior.get("pdemodel") not in ("shiftedlaplace_fd", "shiftedlaplace_fem") or model not in ("constant",
                                                                                                  "periodic"):
        raise NotImplementedError("the GPU sampling path takes the shifted-Laplace FD or FEM prior with a constant "
                                  "or periodic correlation length")
    Lambda = float(root["constantcorrelationlengthmodel"]["Lambda"]) if model == "constant" else 0.0
    cfg = RunConfig(dim=dim, shape=shape, operator=operator, Lambda=Lambda, multigrid=root["multigrid"],
                    smoother=root.get("smoother", {}), sampling=root.get("sampling", {}),
                    measurements=root.get("measurements", {}), correlation=model,
                    pdemodel=prior.get("pdemodel", "shiftedlaplace_fd"))
    if model == "periodic":  # parameters.cc:236-256
        per = root["periodiccorrelationlengthmodel"]
        cfg.Lambda_min, cfg.Lambda_max = float(per["Lambda_min"]), float(per["Lambda_max"])
        if not (cfg.Lambda_max >= cfg.Lambda_min and cfg.Lambda_min > 0):
            raise ValueError("periodic correlation length needs 0 < Lambda_min <= Lambda_max")
    if operator == "posterior":
        path = measurements_file or cfg.measurements["filename"]
        if not os.path.exists(path):
            path = os.path.join(os.path.dirname(os.path.abspath(parameters_file)), path)
        cfg.measurement_data = _read(path)
        if int(cfg.measurement_data["dim"]) != dim:
            raise ValueError("measurement file and parameters disagree on the dimension")
    return cfg
