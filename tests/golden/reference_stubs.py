"""Stand-ins for the reference's un-vendored dependencies (test infrastructure).

Just enough of arraycontext, grudge, meshmode and pytools to import
``actx_dgfem_suite/equations/wave.py`` and ``euler.py`` from a checkout of
the reference and run their own code on NumPy data: the problem set-up
functions (``bump``, ``acoustic_pulse_condition``) and ``wave_operator`` with
its ``wave_flux``.  The grudge operators behind ``wave_operator``
(``weak_local_div`` / ``weak_local_grad``, ``face_mass``, ``inverse_mass``,
traces) are the oracle's (``oracle.rhs``), so a run checks the reference's
composition of them -- signs, flux, boundary pair, which terms meet which
operator -- against the oracle's restatement and the product, with grudge's
trace conventions (``avg = (int + ext) / 2``, ``diff = ext - int``).

Used only by ``tests/golden/make_reference_equations.py`` and
``make_reference_flop_counts.py``, in a container that has the reference
checkout; the fixtures they write travel instead.

Operation counting (``counting()``): every arithmetic operation on DOF
arrays adds the number of output elements, as the reference's FLOP counter
counts its DAG's pointwise nodes (``actx_dgfem_suite/perf_analysis.py:250-377``),
under the domain of its operands: ``"vol"`` (volume nodes), ``"bdry"``
(traces on the boundary faces), ``"int"`` (interior-face trace pairs) or
``"all"`` (the all-faces fluxes), the domain a DOF inherits from the
projection or trace that made it.  The grudge operators (stand-ins over the
oracle) are not counted here; their einsums are counted by the einsum rule.
"""

from __future__ import annotations

import dataclasses
import operator
import sys
import types

import numpy as np


def objarr(items) -> np.ndarray:
    out = np.empty(len(items), dtype=object)
    for i, x in enumerate(items):
        out[i] = x
    return out


def _is_obj(x) -> bool:
    return isinstance(x, np.ndarray) and x.dtype == object


#: operation counts by domain while ``counting()`` is active, else None
COUNTS = None


class counting:
    """Context manager: count DOF operations into a fresh ``COUNTS`` dict."""

    def __enter__(self):
        global COUNTS
        COUNTS = {}
        return COUNTS

    def __exit__(self, *exc):
        global COUNTS
        COUNTS = None


def _count(dom, out):
    if COUNTS is not None:
        key = dom or ("vol" if out.ndim == 2 else "all")
        COUNTS[key] = COUNTS.get(key, 0) + out.size


class DOF:
    """A DOFArray stand-in: one NumPy array (volume (Nel, Np) or faces
    (Nel, 4, Nfp)).  Object arrays broadcast over it element by element.
    ``dom``: the face domain the array lives on (None: volume or neutral)."""

    __array_ufunc__ = None   # NumPy defers to the reflected operators below

    def __init__(self, a, actx=None, dom=None):
        self.a = np.asarray(a, dtype=np.float64)
        self.array_context = actx
        self.dom = dom

    def _bin(self, other, op, swap=False):
        if _is_obj(other) or (isinstance(other, np.ndarray) and other.ndim >= 1):
            return objarr([self._bin(o, op, swap) for o in other])
        o = other.a if isinstance(other, DOF) else other
        odom = other.dom if isinstance(other, DOF) else None
        dom = self.dom or odom
        if self.dom and odom and self.dom != odom:
            dom = "all"
        out = op(o, self.a) if swap else op(self.a, o)
        _count(dom, out)
        return DOF(out, self.array_context, dom)

    def __add__(self, o): return self._bin(o, operator.add)
    def __radd__(self, o): return self._bin(o, operator.add, True)
    def __sub__(self, o): return self._bin(o, operator.sub)
    def __rsub__(self, o): return self._bin(o, operator.sub, True)
    def __mul__(self, o): return self._bin(o, operator.mul)
    def __rmul__(self, o): return self._bin(o, operator.mul, True)
    def __truediv__(self, o): return self._bin(o, operator.truediv)
    def __rtruediv__(self, o): return self._bin(o, operator.truediv, True)
    def __pow__(self, o): return self._bin(o, operator.pow)
    def __neg__(self):
        _count(self.dom, self.a)
        return DOF(-self.a, self.array_context, self.dom)


def cmap(f, x):
    """Apply ``f`` to every DOF of a container (dataclass, object array)."""
    if isinstance(x, DOF):
        return f(x)
    if _is_obj(x):
        return objarr([cmap(f, e) for e in x])
    if dataclasses.is_dataclass(x):
        return type(x)(**{fl.name: cmap(f, getattr(x, fl.name))
                          for fl in dataclasses.fields(x)})
    return x


class _NP:
    """``actx.np``."""
    @staticmethod
    def exp(x): return cmap(lambda d: DOF(np.exp(d.a), d.array_context, d.dom), x)

    @staticmethod
    def sqrt(x):
        def f(d):
            _count(d.dom, d.a)
            return DOF(np.sqrt(d.a), d.array_context, d.dom)
        return cmap(f, x)
    @staticmethod
    def real(x): return x


class StubActx:
    np = _NP()

    def thaw(self, x): return x
    def freeze_thaw(self, x): return x


class DOFDesc:
    def __init__(self, domain_tag, discretization_tag=None):
        self.domain_tag = domain_tag
        self.discretization_tag = discretization_tag

    def with_discr_tag(self, tag): return DOFDesc(self.domain_tag, tag)
    def with_domain_tag(self, tag): return DOFDesc(tag, self.discretization_tag)


def as_dofdesc(x):
    return x if isinstance(x, DOFDesc) else DOFDesc(x)


class _BTagAll:
    def __repr__(self): return "BTAG_ALL"


BTAG_ALL = _BTagAll()
INT_FACES = "int_faces"


class TracePair:
    """grudge's TracePair: ``int``, ``ext``, ``avg``, ``diff`` (= ext - int) and
    attribute access to the fields of container-valued pairs."""

    def __class_getitem__(cls, item):
        return cls

    def __init__(self, dd, *, interior, exterior):
        self.dd = dd
        self.int = interior
        self.ext = exterior

    @property
    def avg(self): return 0.5 * (self.int + self.ext)

    @property
    def diff(self): return self.ext - self.int

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return TracePair(self.dd, interior=getattr(self.int, name),
                         exterior=getattr(self.ext, name))


class StubDcoll:
    """A discretisation collection over an oracle discretisation ``d``."""

    def __init__(self, d, actx):
        self._d = d
        self._actx = actx
        self.dim = d.nodes.shape[0]          # 3 (tetrahedra) or 2 (triangles)

    def nodes(self):
        return objarr([DOF(self._d.nodes[x], self._actx) for x in range(self.dim)])

    def zeros(self, actx):
        return DOF(np.zeros(self._d.nodes.shape[1:]), actx)


def _build_op():
    from oracle import rhs as orc
    op = types.ModuleType("grudge.op")

    def _trace(d, a, idx):
        return a.reshape(-1)[idx]

    def project(dcoll, src, tgt, x):
        d = dcoll._d
        src, tgt = as_dofdesc(src), as_dofdesc(tgt)
        if src.domain_tag == "vol" and tgt.domain_tag == "vol":
            return x
        if src.domain_tag == "vol":          # volume -> boundary faces: traces
            return cmap(lambda z: DOF(_trace(d, z.a, d.int_idx), z.array_context,
                                      "bdry"), x)
        if tgt.domain_tag == "all_faces":    # a face domain into all faces
            keep = d.bdry if src.domain_tag is BTAG_ALL else ~d.bdry
            return cmap(lambda z: DOF(z.a * keep[..., None], z.array_context, "all"), x)
        if tgt.domain_tag == src.domain_tag:  # same faces, another quadrature tag
            return x
        raise NotImplementedError((src.domain_tag, tgt.domain_tag))

    def bdry_trace_pair(dcoll, dd, interior, exterior):
        return TracePair(as_dofdesc(dd), interior=interior, exterior=exterior)

    def interior_trace_pairs(dcoll, w, comm_tag=None):
        d = dcoll._d
        return [TracePair(DOFDesc(INT_FACES),
                          interior=cmap(lambda z: DOF(_trace(d, z.a, d.int_idx), dom="int"), w),
                          exterior=cmap(lambda z: DOF(_trace(d, z.a, d.ext_idx), dom="int"), w))]

    def inverse_mass(dcoll, x):
        return cmap(lambda z: DOF(orc.inverse_mass(dcoll._d, z.a)), x)

    def weak_local_div(dcoll, dd, v):
        return DOF(orc.weak_div(dcoll._d, np.stack([e.a for e in v])))

    def weak_local_grad(dcoll, dd, u):
        g = orc.weak_grad(dcoll._d, u.a)
        return objarr([DOF(g[x]) for x in range(dcoll.dim)])

    def face_mass(dcoll, dd, x):
        return cmap(lambda z: DOF(orc.face_mass(dcoll._d, z.a)), x)

    for f in (project, bdry_trace_pair, interior_trace_pairs, inverse_mass,
              weak_local_div, weak_local_grad, face_mass):
        setattr(op, f.__name__, f)
    return op


def _container_arithmetic(**kw):
    def deco(cls):
        def binop(fn, swap=False):
            def f(self, other):
                if isinstance(other, cls):
                    vals = {fl.name: fn(getattr(self, fl.name), getattr(other, fl.name))
                            for fl in dataclasses.fields(cls)}
                else:
                    vals = {fl.name: (fn(other, getattr(self, fl.name)) if swap
                                      else fn(getattr(self, fl.name), other))
                            for fl in dataclasses.fields(cls)}
                return cls(**vals)
            return f
        cls.__add__ = binop(operator.add)
        cls.__radd__ = binop(operator.add, True)
        cls.__sub__ = binop(operator.sub)
        cls.__mul__ = binop(operator.mul)
        cls.__rmul__ = binop(operator.mul, True)
        cls.__neg__ = lambda self: cls(**{fl.name: -getattr(self, fl.name)
                                          for fl in dataclasses.fields(cls)})
        return cls
    return deco


@dataclasses.dataclass
class ConservedEulerField:
    mass: object
    energy: object
    momentum: object


class _Generic:
    """A placeholder type usable in annotations (``X[...]``, ``X | None``)."""

    def __class_getitem__(cls, item):
        return cls


def install() -> None:
    """Register the stand-in modules in ``sys.modules``."""
    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    generic = lambda name: type(name, (_Generic,), {})  # noqa: E731
    mod("arraycontext", Array=generic("Array"), ArrayContext=generic("ArrayContext"),
        dataclass_array_container=lambda cls: cls,
        with_container_arithmetic=_container_arithmetic)
    grudge = mod("grudge", DiscretizationCollection=generic("DiscretizationCollection"))
    geometry = mod("grudge.geometry")
    geometry.normal = lambda actx, dcoll, dd: objarr(
        [DOF(np.broadcast_to(dcoll._d.normal[..., x][..., None],
                             dcoll._d.int_idx.shape).copy()) for x in range(dcoll.dim)])
    grudge.geometry = geometry
    op = _build_op()
    sys.modules["grudge.op"] = op
    grudge.op = op
    mod("grudge.discretization", DiscretizationCollection=generic("DiscretizationCollection"),
        make_discretization_collection=None)
    mod("grudge.dof_desc", DISCR_TAG_BASE="base", DISCR_TAG_QUAD="quad",
        DiscretizationTag=generic("DiscretizationTag"), DOFDesc=DOFDesc,
        as_dofdesc=as_dofdesc)
    mod("grudge.trace_pair", TracePair=TracePair)
    mod("grudge.models")
    mod("grudge.models.euler", ConservedEulerField=ConservedEulerField,
        EulerOperator=None, InviscidWallBC=None)
    mod("meshmode")
    mod("meshmode.dof_array", DOFArray=generic("DOFArray"))
    mod("meshmode.mesh", BTAG_ALL=BTAG_ALL)
    mod("meshmode.mesh.generation", generate_regular_rect_mesh=None)
    mod("meshmode.discretization")
    mod("meshmode.discretization.poly_element", QuadratureSimplexGroupFactory=None,
        default_simplex_group_factory=None)
    mod("pytools")
    mod("pytools.obj_array", flat=objarr, new_1d=objarr,
        ObjectArray=generic("ObjectArray"))
