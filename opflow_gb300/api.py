"""Python mirror of OpFlow's user-facing API for the two accelerated paths.

Names, argument meanings and error behaviour follow the reference (paths relative to the OpFlow tree):

  MeshBuilder(CartesianMesh).newMesh(...).setMeshOfDim(d, min, max).build()
                                   -> src/Core/Mesh/Structured/CartesianMesh.hpp:122-305
  ExprBuilder().setMesh(m).setBC(d, DimPos.start, BCType.Dirc, v).setLoc(..).setExt(..).build()
                                   -> src/Core/Field/MeshBased/Structured/CartesianField.hpp:796-1033
  u.assign(u + dt * a * (d2x(u) + d2y(u)))        ( C++: u = u + dt*a*(d2x<D2SecondOrderCentered>(u) + ...) )
                                   -> src/Core/Loops/FieldAssigner.hpp:27-84
  Solve(lambda e: f == d2x(e) + d2y(e), p, params) / makeEqnSolveHandler(...)
                                   -> src/Core/Equation/UnifiedSolve.hpp:36-43, HYPREEqnSolveHandler.hpp:44-48

Python cannot overload `=`, so `u = expr` is spelled `u.assign(expr)` (and `u += expr` is
`u.assign(expr, op="+")`).  Every call goes through the C ABI of libopflow_gpu.so.
"""
import atexit
import ctypes as C
import os
import threading

import numpy as np

from . import _capi as capi
from ._capi import check, lib


class LocOnMesh:
    Corner = capi.CORNER
    Center = capi.CENTER


class BCType:
    Undefined = capi.BC_UNDEFINED
    Dirc = capi.BC_DIRC
    Neum = capi.BC_NEUM
    Periodic = capi.BC_PERIODIC
    Symm = capi.BC_SYMM
    ASymm = capi.BC_ASYMM


class DimPos:
    start = 0
    end = 1


# ---------------------------------------------------------------------------------------------- context
_ctx_lock = threading.Lock()
_default_ctx = {}
_exiting = [False]


@atexit.register
def _mark_exit():
    # at interpreter shutdown objects are finalised in no particular order; device memory is released
    # with the process instead of through destructors that may outlive their context
    _exiting[0] = True


class Context:
    """One device + one CUDA stream (opflow_ctx)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        check(lib().opflow_ctx_create(device, C.byref(h)))
        self.handle = h
        self.device = device

    def synchronize(self):
        check(lib().opflow_ctx_synchronize(self.handle))

    def set_stream(self, stream_ptr):
        check(lib().opflow_ctx_set_stream(self.handle, C.c_void_p(stream_ptr)))

    def close(self):
        if self.handle and not _exiting[0]:
            lib().opflow_ctx_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_context(device=0):
    with _ctx_lock:
        if device not in _default_ctx:
            _default_ctx[device] = Context(device)
        return _default_ctx[device]


# ------------------------------------------------------------------------------------------------- mesh
class CartesianMesh:
    def __init__(self, ndim, dims, start, pad_width, x, dx):
        self.ndim = ndim
        self.dims = list(dims)
        self.start = list(start)
        self.pad_width = pad_width
        self.x = [np.ascontiguousarray(v, dtype=np.float64) for v in x]
        self.dx = [np.ascontiguousarray(v, dtype=np.float64) for v in dx]

    def desc(self):
        d = capi.MeshDesc()
        d.ndim = self.ndim
        for k in range(self.ndim):
            d.dims[k] = self.dims[k]
            d.start[k] = self.start[k]
            d.x[k] = self.x[k].ctypes.data_as(C.POINTER(C.c_double))
            d.dx[k] = self.dx[k].ctypes.data_as(C.POINTER(C.c_double))
        d.pad_width = self.pad_width
        d._keep = (self.x, self.dx)
        return d

    def getDims(self):
        return list(self.dims)

    def x_at(self, d, i):
        return self.x[d][i - (self.start[d] - self.pad_width)]

    def dx_at(self, d, i):
        return self.dx[d][i - (self.start[d] - self.pad_width)]


class MeshBuilder:
    """MeshBuilder<CartesianMesh<Meta::int_<ndim>>>; padding width 5 and start 0 by default."""

    def __init__(self, ndim=None):
        self._ndim = ndim
        self._dims = None
        self._pad = 5
        self._start = None
        self._minmax = {}

    def newMesh(self, *dims):
        self._dims = [int(v) for v in dims]
        if self._ndim is None:
            self._ndim = len(self._dims)
        if len(self._dims) != self._ndim:
            raise ValueError("newMesh got %d extents for a %d-D mesh" % (len(self._dims), self._ndim))
        return self

    def setPadWidth(self, w):
        self._pad = int(w)
        return self

    def setStart(self, s):
        self._start = [int(v) for v in s]
        return self

    def setMeshOfDim(self, k, vmin, vmax):
        self._minmax[int(k)] = (float(vmin), float(vmax))
        return self

    def build(self):
        if self._dims is None:
            raise ValueError("newMesh() was not called")
        start = self._start or [0] * self._ndim
        xs, dxs = [], []
        for k in range(self._ndim):
            n = self._dims[k] + 2 * self._pad
            x = np.zeros(n)
            dx = np.zeros(n - 1)
            lo, hi = self._minmax.get(k, (0.0, 1.0))
            check(lib().opflow_mesh_uniform(self._dims[k], start[k], self._pad, lo, hi,
                                            x.ctypes.data_as(C.POINTER(C.c_double)),
                                            dx.ctypes.data_as(C.POINTER(C.c_double))))
            xs.append(x)
            dxs.append(dx)
        return CartesianMesh(self._ndim, self._dims, start, self._pad, xs, dxs)


# ------------------------------------------------------------------------------------------ expressions
class Expr:
    """Base of every expression node; arithmetic builds trees (Expression<Op, Args...>)."""

    def __add__(self, o):
        return ExprNode(capi.NODE_ADD, self, _wrap(o))

    def __radd__(self, o):
        return ExprNode(capi.NODE_ADD, _wrap(o), self)

    def __sub__(self, o):
        return ExprNode(capi.NODE_SUB, self, _wrap(o))

    def __rsub__(self, o):
        return ExprNode(capi.NODE_SUB, _wrap(o), self)

    def __mul__(self, o):
        return ExprNode(capi.NODE_MUL, self, _wrap(o))

    def __rmul__(self, o):
        return ExprNode(capi.NODE_MUL, _wrap(o), self)

    def __truediv__(self, o):
        return ExprNode(capi.NODE_DIV, self, _wrap(o))

    def __rtruediv__(self, o):
        return ExprNode(capi.NODE_DIV, _wrap(o), self)

    def __neg__(self):
        return ExprNode(capi.NODE_NEG, self)

    def __eq__(self, o):  # lhs == rhs -> Equation (Equation.hpp:41-55)
        return Equation(self, _wrap(o))

    # comparisons (Logical/Compare.hpp); `==` stays the equation builder, as in the reference
    def __gt__(self, o):
        return ExprNode(capi.NODE_GT, self, _wrap(o))

    def __ge__(self, o):
        return ExprNode(capi.NODE_GE, self, _wrap(o))

    def __lt__(self, o):
        return ExprNode(capi.NODE_LT, self, _wrap(o))

    def __le__(self, o):
        return ExprNode(capi.NODE_LE, self, _wrap(o))

    def __ne__(self, o):
        return ExprNode(capi.NODE_NE, self, _wrap(o))

    # && / || / ! of Logical/Boolean.hpp, spelled & | ~ in Python
    def __and__(self, o):
        return ExprNode(capi.NODE_AND, self, _wrap(o))

    def __rand__(self, o):
        return ExprNode(capi.NODE_AND, _wrap(o), self)

    def __or__(self, o):
        return ExprNode(capi.NODE_OR, self, _wrap(o))

    def __ror__(self, o):
        return ExprNode(capi.NODE_OR, _wrap(o), self)

    def __invert__(self):
        return ExprNode(capi.NODE_NOT, self)

    def __abs__(self):
        return ExprNode(capi.NODE_FUNC1, self, param=capi.FUNC1["abs"])

    def __hash__(self):
        return id(self)


class ScalarExpr(Expr):
    def __init__(self, v):
        self.value = float(v)


def _wrap(o):
    if isinstance(o, Expr):
        return o
    if isinstance(o, (int, float, np.floating, np.integer)):
        return ScalarExpr(o)
    raise TypeError("cannot use %r in an expression" % (o,))


class ExprNode(Expr):
    def __init__(self, kind, a=None, b=None, dim=0, c=None, param=0):
        self.kind, self.a, self.b, self.dim, self.c, self.param = kind, a, b, dim, c, param


class Equation:
    """`lhs == rhs` (Equation.hpp:27-55); the solver works on the tree of `lhs - rhs`."""

    def __init__(self, lhs, rhs):
        self.lhs, self.rhs = lhs, rhs

    def residual_expr(self):
        return ExprNode(capi.NODE_SUB, self.lhs, self.rhs)


def Eq(lhs, rhs):
    """`lhs == rhs` with the operands kept in this order even when lhs is a plain number (Python
    would otherwise reflect `1.0 == expr` into `expr == 1.0`)."""
    return Equation(_wrap(lhs), _wrap(rhs))


# Kernel tags with the reference's names, for dx(u, D1FirstOrderBiasedDownwind) in the place of
# dx<D1FirstOrderBiasedDownwind>(u) (DiffsInterface.hpp).
D2SecondOrderCentered = capi.NODE_D2
D1FirstOrderCentered = capi.NODE_D1
D1FirstOrderBiasedUpwind = capi.NODE_D1_BIASED_UP
D1FirstOrderBiasedDownwind = capi.NODE_D1_BIASED_DOWN
D1WENO53Upwind = capi.NODE_WENO53_UP
D1WENO53Downwind = capi.NODE_WENO53_DOWN


def _diff(kind, dim):
    def f(e, kernel=None):
        return ExprNode(kind if kernel is None else kernel, _wrap(e), None, dim)
    return f


# D2SecondOrderCentered<d> (DiffsInterface.hpp:47)
def d2(e, dim):
    return ExprNode(capi.NODE_D2, _wrap(e), None, dim)


d2x, d2y, d2z = _diff(capi.NODE_D2, 0), _diff(capi.NODE_D2, 1), _diff(capi.NODE_D2, 2)


# D1FirstOrderCentered<d>: dx/dy/dz<D1FirstOrderCentered>
def d1(e, dim):
    return ExprNode(capi.NODE_D1, _wrap(e), None, dim)


dx, dy, dz = _diff(capi.NODE_D1, 0), _diff(capi.NODE_D1, 1), _diff(capi.NODE_D1, 2)


# d1<D1WENO53Downwind<d>> / d1<D1WENO53Upwind<d>>
def d1_weno53_downwind(e, dim=0):
    return ExprNode(capi.NODE_WENO53_DOWN, _wrap(e), None, dim)


def d1_weno53_upwind(e, dim=0):
    return ExprNode(capi.NODE_WENO53_UP, _wrap(e), None, dim)


# d1<D1FirstOrderBiasedUpwind<d>> / d1<D1FirstOrderBiasedDownwind<d>>: one-sided first differences
# (D1FirstOrderBiasedUpwind.hpp:53-58, D1FirstOrderBiasedDownwind.hpp:52-57); the reference's
# examples/CONV1D writes the downwind one as dx<D1FirstOrderBiasedDownwind>(u).
def d1_biased_upwind(e, dim=0):
    return ExprNode(capi.NODE_D1_BIASED_UP, _wrap(e), None, dim)


def d1_biased_downwind(e, dim=0):
    return ExprNode(capi.NODE_D1_BIASED_DOWN, _wrap(e), None, dim)


# d1IntpCenterToCorner<d> (IntpInterface.hpp:22-33, D1Linear Cen2Cor)
def d1IntpCenterToCorner(e, dim):
    return ExprNode(capi.NODE_INTP_C2C, _wrap(e), None, dim)


# d1IntpCornerToCenter<d> (IntpInterface.hpp:31-34, D1Linear Cor2Cen: the midpoint of e(i), e(i+1))
def d1IntpCornerToCenter(e, dim):
    return ExprNode(capi.NODE_INTP_COR2CEN, _wrap(e), None, dim)


# conditional(c, a, b) = c ? a : b (Conditional.hpp)
def conditional(c, a, b):
    return ExprNode(capi.NODE_COND, _wrap(c), _wrap(a), c=_wrap(b))


def logical_and(a, b):
    return ExprNode(capi.NODE_AND, _wrap(a), _wrap(b))


def logical_or(a, b):
    return ExprNode(capi.NODE_OR, _wrap(a), _wrap(b))


def logical_not(a):
    return ExprNode(capi.NODE_NOT, _wrap(a))


def _func1(name):
    fid = capi.FUNC1[name]

    def f(e):
        return ExprNode(capi.NODE_FUNC1, _wrap(e), param=fid)
    f.__name__ = name
    f.__doc__ = "Per-element std::%s (Arithmetic/AMDS.hpp)." % name
    return f


def _func2(name):
    fid = capi.FUNC2[name]

    def f(a, b):
        return ExprNode(capi.NODE_FUNC2, _wrap(a), _wrap(b), param=fid)
    f.__name__ = name
    f.__doc__ = "Per-element std::%s (Arithmetic/AMDS.hpp, MinMax.hpp)." % name
    return f


_FUNCS = {**{n: _func1(n) for n in capi.FUNC1}, **{n: _func2(n) for n in capi.FUNC2}}


def __getattr__(name):
    """api.max, api.sqrt, ... (module attributes only, so that this module's own code keeps Python's
    builtin max / min / abs / round / pow)."""
    try:
        return _FUNCS[name]
    except KeyError:
        raise AttributeError("module %r has no attribute %r" % (__name__, name)) from None


# Flux-limiter interpolators of D1FluxLimiterBasedIntpOp.hpp: d1Intp<D1QUICK, d, Cen2Cor>(u, e) is
# d1IntpCenterToCorner(e, d, limiter="QUICK", u=u): e interpolated to the faces along d, upwinded by
# the sign of u at the face (D1FluxLimiter.hpp:136-201).
FLUX_LIMITERS = {"Central": capi.FL_CDS, "QUICK": capi.FL_QUICK, "CUI": capi.FL_CUI, "Fromm": capi.FL_FROMM,
                 "LinearUpwind": capi.FL_LUI, "Minmod": capi.FL_MINMOD, "Superbee": capi.FL_SUPERBEE,
                 "MUSCL": capi.FL_MUSCL, "Harmonic": capi.FL_HARMONIC, "Albada": capi.FL_VANALBADA,
                 "UMIST": capi.FL_UMIST, "SPL13": capi.FL_SPL13, "SPLMax12": capi.FL_SPLMAX12,
                 "SPLMax13": capi.FL_SPLMAX13, "KorenLimitedCUI": capi.FL_KOREN, "SMART": capi.FL_SMART,
                 "BSOU": capi.FL_BSOU}


def d1_flux_limiter_intp(u, e, dim, limiter, to_corner=True):
    """d1Intp<D1FluxLimiterGen<K>::Op, dim, Cen2Cor or Cor2Cen>(u, e)."""
    k = FLUX_LIMITERS[limiter] if isinstance(limiter, str) else int(limiter)
    kind = capi.NODE_INTP_FL_CEN2COR if to_corner else capi.NODE_INTP_FL_COR2CEN
    return ExprNode(kind, _wrap(u), _wrap(e), dim, param=k)


def serialize(expr, extra_leaves=()):
    """Postfix node list (children first, root last) and the ordered leaf fields."""
    nodes = []
    leaves = list(extra_leaves)
    memo = {}

    def leaf_slot(f):
        for i, g in enumerate(leaves):
            if g is f:
                return i
        leaves.append(f)
        return len(leaves) - 1

    def rec(e):
        key = id(e)
        is_leaf = getattr(e, "_is_field", False)
        if key in memo and not is_leaf:
            return memo[key]
        if is_leaf:
            n = (capi.NODE_FIELD, -1, -1, 0, leaf_slot(e), 0.0, -1)
        elif isinstance(e, ScalarExpr):
            n = (capi.NODE_CONST, -1, -1, 0, 0, e.value, -1)
        elif isinstance(e, ExprNode):
            a = rec(e.a) if e.a is not None else -1
            b = rec(e.b) if e.b is not None else -1
            c = rec(e.c) if getattr(e, "c", None) is not None else -1
            n = (e.kind, a, b, e.dim, getattr(e, "param", 0), 0.0, c)
        else:
            raise TypeError("not an expression: %r" % (e,))
        nodes.append(n)
        memo[key] = len(nodes) - 1
        return len(nodes) - 1

    rec(_wrap(expr))
    arr = (capi.Node * len(nodes))()
    for i, (k, a, b, d, f, v, c) in enumerate(nodes):
        arr[i].kind, arr[i].a, arr[i].b, arr[i].dim, arr[i].field, arr[i].value, arr[i].c = k, a, b, d, f, v, c
    return arr, leaves


# ------------------------------------------------------------------------------------------------ field
_ARITH = {"=": capi.ASSIGN_EQ, "+": capi.ASSIGN_ADD, "-": capi.ASSIGN_SUB, "*": capi.ASSIGN_MUL, "/": capi.ASSIGN_DIV}
_MODES = {"exact": capi.EVAL_EXACT, "fast": capi.EVAL_FAST}


class CartesianField(Expr):
    """CartesianField<Real, CartesianMesh<Dim>> whose data lives in HBM."""

    _is_field = True

    def __init__(self, mesh, desc, ctx, name="field"):
        self.mesh = mesh
        self.desc = desc
        self.ctx = ctx
        self.name = name
        h = C.c_void_p()
        md = mesh.desc()
        check(lib().opflow_field_create(ctx.handle, C.byref(md), C.byref(desc), C.byref(h)))
        self.handle = h
        info = capi.FieldInfo()
        check(lib().opflow_field_get_info(h, C.byref(info)))
        self.info = info

    # ---- ranges (CartesianField / StructuredFieldExpr members) ----
    def _rng(self, which):
        r = getattr(self.info, which)
        return [(r[d][0], r[d][1]) for d in range(self.info.ndim)]

    @property
    def assignableRange(self):
        return self._rng("assignable")

    @property
    def accessibleRange(self):
        return self._rng("accessible")

    @property
    def logicalRange(self):
        return self._rng("logical")

    @property
    def localRange(self):
        return self._rng("local")

    @property
    def padding(self):
        return self.info.padding

    @property
    def shape(self):
        """numpy shape of the full data array (z, y, x order; x fastest)."""
        D = self.info.ndim
        return tuple(self.info.data_dims[d] for d in reversed(range(D)))

    @property
    def offset(self):
        return [self.info.data_offset[d] for d in range(self.info.ndim)]

    # ---- data movement ----
    def download(self):
        a = np.empty(self.info.count, dtype=np.float64)
        check(lib().opflow_field_download(self.handle, a.ctypes.data_as(C.POINTER(C.c_double)), a.size))
        return a.reshape(self.shape)

    def upload(self, arr, update_padding=True):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(-1)
        check(lib().opflow_field_upload(self.handle, a.ctypes.data_as(C.POINTER(C.c_double)), a.size))
        if update_padding:
            self.updatePadding()

    def updatePadding(self):
        check(lib().opflow_field_update_padding(self.handle))

    def device_ptr(self):
        p = C.c_void_p()
        check(lib().opflow_field_device_ptr(self.handle, C.byref(p)))
        return p.value

    def index_slices(self, ranges):
        """numpy slices (z, y, x order) of the data array covering the given index ranges."""
        D = self.info.ndim
        sl = []
        for d in reversed(range(D)):
            lo, hi = ranges[d]
            o = self.info.data_offset[d]
            sl.append(slice(lo - o, hi - o))
        return tuple(sl)

    # ---- assignment ----
    def assign(self, expr, op="=", mode="exact", steps=1):
        """`self <op>= expr` (Expr::operator=, +=, ... through FieldAssigner::assign), `steps` times.

        mode "exact": the reference's IEEE operations in its order (bit-identical); "fast": a linear
        constant-coefficient stencil of one field in exact 64-bit fixed point (within 1e-14).  In fast
        mode, `steps` >= 2 FTCS steps of a Dirichlet node grid without a ghost layer, with weights that
        keep the maximum principle, run resident: the field stays in fixed point between the steps (3D
        steady-state steps stage their planes in shared memory by TMA; long 2D runs replay a CUDA graph).
        """
        if isinstance(expr, (int, float)):
            check(lib().opflow_field_fill(self.handle, _ARITH[op], float(expr)))
            return self
        if isinstance(expr, CartesianField) and op == "=" and expr is not self:
            if expr.info.count == self.info.count:
                check(lib().opflow_field_copy(self.handle, expr.handle))
                return self
        nodes, leaves = serialize(expr)
        hs = (C.c_void_p * max(1, len(leaves)))(*[f.handle.value for f in leaves])
        check(lib().opflow_assign_repeat(self.ctx.handle, self.handle, _ARITH[op], nodes, len(nodes), hs, len(leaves),
                                         _MODES[mode], int(steps)))
        return self

    def initBy(self, fn):
        """CartesianField::initBy (CartesianField.hpp:282-294): fn(coords) at nodes or cell centres."""
        D = self.info.ndim
        a = self.download()
        rng = [(max(self.info.assignable[d][0], self.info.local[d][0]), min(self.info.assignable[d][1], self.info.local[d][1]))
               for d in range(D)]
        grids = []
        for d in range(D):
            idx = np.arange(rng[d][0], rng[d][1])
            x = np.array([self.mesh.x_at(d, i) for i in idx])
            if self.desc.loc[d] == capi.CENTER:
                x = x + .5 * np.array([self.mesh.dx_at(d, i) for i in idx])
            grids.append(x)
        mesh = np.meshgrid(*grids, indexing="ij")
        vals = np.asarray(fn(mesh), dtype=np.float64)
        a[self.index_slices(rng)] = np.transpose(vals) if D > 1 else vals
        self.upload(a)
        return self

    def close(self):
        if getattr(self, "handle", None) and not _exiting[0]:
            lib().opflow_field_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ExprBuilder:
    """ExprBuilder<CartesianField<Real, Mesh>>."""

    def __init__(self):
        self._mesh = None
        self._name = "field"
        self._loc = None
        self._bc = {}
        self._ext = {}
        self._padding = 0

    def setName(self, n):
        self._name = n
        return self

    def setMesh(self, m):
        self._mesh = m
        return self

    def setLoc(self, loc):
        if isinstance(loc, (list, tuple)):
            self._loc = list(loc)
        else:
            self._loc = loc
        return self

    def setLocOfDim(self, d, loc):
        if not isinstance(self._loc, list):
            self._loc = [self._loc if self._loc is not None else LocOnMesh.Corner] * 3
        self._loc[d] = loc
        return self

    def setBC(self, d, pos, bctype, value=0.0):
        self._bc[(d, pos)] = (bctype, float(value))
        return self

    def setExt(self, *args):
        if len(args) == 1:
            for d in range(3):
                self._ext[(d, 0)] = self._ext[(d, 1)] = int(args[0])
        else:
            d, pos, w = args
            self._ext[(d, pos)] = int(w)
        return self

    def setPadding(self, p):
        self._padding = int(p)
        return self

    def desc(self):
        if self._mesh is None:
            raise ValueError("setMesh() was not called")
        D = self._mesh.ndim
        fd = capi.FieldDesc()
        fd.ndim = D
        loc = self._loc
        for d in range(D):
            fd.loc[d] = loc[d] if isinstance(loc, list) else (loc if loc is not None else LocOnMesh.Corner)
            for s in range(2):
                t, v = self._bc.get((d, s), (BCType.Undefined, 0.0))
                fd.bc_type[d][s] = t
                fd.bc_value[d][s] = v
                fd.ext[d][s] = self._ext.get((d, s), 0)
        fd.padding = self._padding
        return fd

    def build(self, ctx=None):
        return CartesianField(self._mesh, self.desc(), ctx or default_context(), self._name)


# ------------------------------------------------------------------------------------------ snapshots
class TimeStamp:
    """Utils::TimeStamp (src/Utils/Writers/Streams.hpp:31-45)."""

    def __init__(self, time=0.0, step=None):
        self.time, self.step = float(time), step


class RawBinaryOStream:
    """Utils::RawBinaryOStream (src/Utils/Writers/RawBinaryStream.hpp:42-62, 97-150): `stream << TimeStamp(t)`
    sets the time, `stream << field` writes <dir>/<name>_<count>.cart and advances the counter.  As in
    the reference, the files go to the directory part of `path` (its parent)."""

    def __init__(self, path):
        self.dir = os.path.dirname(os.fspath(path)) or "."
        self.time = 0.0
        self.count = 0

    def setCounterTo(self, c):
        self.count = int(c)

    def __lshift__(self, x):
        if isinstance(x, TimeStamp):
            self.time = x.time
            return self
        check(lib().opflow_field_write_raw(x.handle, self.dir.encode(), x.name.encode(), self.count, self.time))
        self.count += 1
        return self


class RawBinaryIStream:
    """Utils::RawBinaryIStream (RawBinaryStream.hpp:64-77, 152-224): `stream >> field` reads
    <dir>/<name>_<count>.cart into the field (mesh and ranges checked) and advances the counter; the
    time stamp read is kept in `time`."""

    def __init__(self, path):
        self.dir = os.path.dirname(os.fspath(path)) or "."
        self.count = 0
        self.time = 0.0

    def setCounterTo(self, c):
        self.count = int(c)

    def __rshift__(self, f):
        t = C.c_double(0.0)
        check(lib().opflow_field_read_raw(f.handle, self.dir.encode(), f.name.encode(), self.count, C.byref(t)))
        self.time = t.value
        self.count += 1
        return self


def describe(mesh, desc):
    """Ranges ExprBuilder::build computes, without touching a GPU (opflow_field_describe)."""
    info = capi.FieldInfo()
    md = mesh.desc()
    check(lib().opflow_field_describe(C.byref(md), C.byref(desc), C.byref(info)))
    return info


# ------------------------------------------------------------------------------------------ implicit path
# StructSolverType (src/Core/Solvers/Struct/StructSolver.hpp:23-34) -> (outer iteration, preconditioner)
STRUCT_SOLVERS = {"PCG": capi.KRYLOV_PCG, "GMRES": capi.KRYLOV_GMRES, "FGMRES": capi.KRYLOV_FGMRES,
                  "LGMRES": capi.KRYLOV_LGMRES, "BICGSTAB": capi.KRYLOV_BICGSTAB}
STRUCT_PRECONDS = {"PFMG": capi.PRECOND_MG, "SMG": capi.PRECOND_MG, "CYCRED": capi.PRECOND_MG,
                   "Jacobi": capi.PRECOND_JACOBI, "None": capi.PRECOND_NONE,
                   # equation sets only: AMGCL's amg<smoothed_aggregation, spai0> (AMGCLEqnSolveHandler.hpp)
                   "AMG": capi.PRECOND_AMG}


class StructSolverParams:
    """StructSolverParamsBase (src/Core/Solvers/Struct/StructSolver.hpp:39-51) with the PFMG knobs
    (StructSolverPFMG.hpp:23-33), the GMRES ones (kDim, absTol) and the GPU extensions (precision form,
    coarse size).  `solver` / `precond` name the StructSolverType pair of
    PrecondStructSolver<solver, precond>; a preconditioner type as `solver` (PFMG, SMG, Jacobi) with
    precond "None" iterates it alone."""

    def __init__(self, tol=1e-10, maxIter=200, staticMat=False, pinValue=False, precision="fp64", preSweeps=2,
                 postSweeps=2, coarseMax=64, zeroGuess=False, solver="PCG", precond="PFMG", kDim=5, absTol=0.0):
        self.tol, self.maxIter, self.staticMat, self.pinValue = tol, maxIter, staticMat, pinValue
        self.precision, self.preSweeps, self.postSweeps, self.coarseMax, self.zeroGuess = (precision, preSweeps, postSweeps,
                                                                                           coarseMax, zeroGuess)
        self.solver, self.precond, self.kDim, self.absTol = solver, precond, kDim, absTol

    def krylov_and_precond(self):
        if self.solver in STRUCT_SOLVERS:
            return STRUCT_SOLVERS[self.solver], STRUCT_PRECONDS[self.precond]
        if self.solver in STRUCT_PRECONDS and self.precond == "None":
            return capi.KRYLOV_NONE, STRUCT_PRECONDS[self.solver]
        raise ValueError("unsupported solver combination %s + %s" % (self.solver, self.precond))

    def to_c(self):
        p = capi.SolveParams()
        p.tol = float(self.tol)
        p.max_iter = int(self.maxIter)
        p.static_mat = int(bool(self.staticMat))
        p.pin_value = int(bool(self.pinValue))
        p.precision = {"fp64": capi.PREC_FP64, "mixed": capi.PREC_MIXED}[self.precision]
        p.pre_sweeps, p.post_sweeps = int(self.preSweeps), int(self.postSweeps)
        p.coarse_max = int(self.coarseMax)
        p.zero_guess = int(bool(self.zeroGuess))
        p.krylov, p.precond = self.krylov_and_precond()
        p.kdim = int(self.kDim)
        p.abs_tol = float(self.absTol)
        return p


class EqnSolveState:
    """EqnSolveState{niter, relerr, abserr} (src/Core/Equation/EqnSolveHandler.hpp:17-25)."""

    def __init__(self, st):
        self.niter = st.iterations
        self.relerr = st.rel_residual
        self.abserr = st.abs_residual
        self.converged = bool(st.converged)
        self.setup_ms = st.setup_ms
        self.solve_ms = st.solve_ms

    def __repr__(self):
        return "EqnSolveState(niter=%d, relerr=%.3g)" % (self.niter, self.relerr)


class EqnSolveHandler:
    """makeEqnSolveHandler(getter, target, PrecondStructSolver<PCG,PFMG>) (HYPREEqnSolveHandler.hpp:44-231):
    `getter(e)` builds the equation in the unknown `e`; the target field is the StencilField's base."""

    def __init__(self, getter, target, params=None):
        self.target = target
        self.params = params or StructSolverParams()
        eq = getter(target)
        if not isinstance(eq, Equation):
            raise TypeError("the equation getter must return `lhs == rhs` (use api.Eq for a scalar lhs)")
        nodes, leaves = serialize(eq.residual_expr(), [target])
        self._leaves = leaves
        hs = (C.c_void_p * len(leaves))(*[f.handle.value for f in leaves])
        p = self.params.to_c()
        h = C.c_void_p()
        check(lib().opflow_solver_create(target.ctx.handle, target.handle, nodes, len(nodes), hs, len(leaves), 0, C.byref(p), C.byref(h)))
        self.handle = h

    def solve(self):
        st = capi.SolveState()
        rc = lib().opflow_solver_solve(self.handle, C.byref(st))
        if rc not in (capi.OK, capi.E_NOT_CONVERGED):
            check(rc)
        return EqnSolveState(st)

    def close(self):
        if getattr(self, "handle", None) and not _exiting[0]:
            lib().opflow_solver_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def makeEqnSolveHandler(getter, target, params=None):
    return EqnSolveHandler(getter, target, params)


def Solve(getter, target, params=None, pparams=None):
    """Solve(f, target, params, pparams) (src/Core/Equation/UnifiedSolve.hpp:36-43): one solve."""
    return EqnSolveHandler(getter, target, params).solve()


class EqnSetSolveHandler:
    """makeEqnSolveHandler over an equation set / SolveEqns (src/Core/Equation/UnifiedSolve.hpp:69-100,
    AMGCLEqnSolveHandler.hpp:53-190): getters[k](*targets) returns equation k, solved for targets[k]
    jointly with the others.  `params` (one StructSolverParams) picks the outer iteration and the
    preconditioner: "AMG" (smoothed aggregation over the whole coupled matrix, AMGCL's
    amg<smoothed_aggregation, spai0>), or a block-diagonal one ("PFMG": each equation's multigrid,
    "Jacobi", "None"); `pins[k]` pins equation k's last unknown (CSRMatrixGenerator)."""

    def __init__(self, getters, targets, params=None, pins=None):
        if len(getters) != len(targets):
            raise ValueError("one getter per target")
        self.targets = list(targets)
        self.params = params or StructSolverParams(solver="BICGSTAB", precond="PFMG")
        leaves = list(targets)
        node_lists = []
        for g in getters:
            eq = g(*targets)
            if not isinstance(eq, Equation):
                raise TypeError("each getter must return `lhs == rhs`")
            nodes, leaves = serialize(eq.residual_expr(), leaves)
            node_lists.append(nodes)
        self._nodes = node_lists
        self._leaves = leaves
        n = len(targets)
        tg = (C.c_void_p * n)(*[t.handle.value for t in targets])
        trees = (C.c_void_p * n)(*[C.cast(nl, C.c_void_p).value for nl in node_lists])
        counts = (C.c_int * n)(*[len(nl) for nl in node_lists])
        lv = (C.c_void_p * len(leaves))(*[f.handle.value for f in leaves])
        pins = pins or [False] * n
        pn = (C.c_int * n)(*[int(bool(p)) for p in pins])
        p = self.params.to_c()
        h = C.c_void_p()
        check(lib().opflow_eqnset_create(targets[0].ctx.handle, n, tg, trees, counts, lv, len(leaves), pn, C.byref(p), C.byref(h)))
        self.handle = h

    def solve(self):
        st = capi.SolveState()
        rc = lib().opflow_eqnset_solve(self.handle, C.byref(st))
        if rc not in (capi.OK, capi.E_NOT_CONVERGED):
            check(rc)
        return EqnSolveState(st)

    def csr(self):
        """The assembled coupled system (CSRMatrixGenerator's numbering): (row_ptr, cols, vals, rhs)."""
        nr, nnz = C.c_longlong(0), C.c_longlong(0)
        check(lib().opflow_eqnset_csr(self.handle, C.byref(nr), C.byref(nnz), None, None, None, None))
        rp = np.zeros(nr.value + 1, dtype=np.int64)
        cols = np.zeros(nnz.value, dtype=np.int64)
        vals = np.zeros(nnz.value)
        rhs = np.zeros(nr.value)
        check(lib().opflow_eqnset_csr(self.handle, C.byref(nr), C.byref(nnz), rp.ctypes.data, cols.ctypes.data, vals.ctypes.data,
                                      rhs.ctypes.data))
        return rp, cols, vals, rhs

    def close(self):
        if getattr(self, "handle", None) and not _exiting[0]:
            lib().opflow_eqnset_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def SolveEqns(getters, targets, params=None, pins=None):
    """SolveEqns(getter_0, ..., targets..., mapper, params): one solve of the coupled set."""
    return EqnSetSolveHandler(getters, targets, params, pins).solve()


def assemble(getter, target, pin=False):
    """The coefficients and right-hand side HYPREEqnSolveHandler::generateAb would hand to HYPRE
    (opflow_assemble): (offsets[n_entries, D], coef[cells, n_entries], rhs[cells])."""
    eq = getter(target)
    nodes, leaves = serialize(eq.residual_expr(), [target])
    hs = (C.c_void_p * len(leaves))(*[f.handle.value for f in leaves])
    ne, nc = C.c_int(0), C.c_size_t(0)
    L = lib()
    check(L.opflow_assemble(target.ctx.handle, target.handle, nodes, len(nodes), hs, len(leaves), 0, int(pin), C.byref(ne), None, None,
                            None, C.byref(nc)))
    D = target.info.ndim
    off = np.zeros(ne.value * D, dtype=np.int32)
    coef = np.zeros(nc.value * ne.value)
    rhs = np.zeros(nc.value)
    check(L.opflow_assemble(target.ctx.handle, target.handle, nodes, len(nodes), hs, len(leaves), 0, int(pin), C.byref(ne),
                            off.ctypes.data_as(C.POINTER(C.c_int)), coef.ctypes.data_as(C.POINTER(C.c_double)),
                            rhs.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nc)))
    return off.reshape(ne.value, D), coef.reshape(nc.value, ne.value), rhs


def weno_rk3(u, dt, steps=1, upwind=False, dim=0, u1=None, u2=None, mode=None):
    """One or more Shu-Osher RK3 steps of u_t + d1<WENO53>(u) = 0 along a periodic dim, fused
    (opflow_weno_rk3_mode); in EXACT mode (the default) identical to the three assignments
        u1 = u - dt*d1<W>(u); u2 = 0.75*u + 0.25*(u1 - dt*d1<W>(u1)); u = 1/3*u + 2/3*(u2 - dt*d1<W>(u2)).
    mode=EvalMode.FAST: contracted arithmetic and one reciprocal for the weights (not bit-identical)."""
    kind = capi.NODE_WENO53_UP if upwind else capi.NODE_WENO53_DOWN
    m = capi.EVAL_EXACT if mode is None else int(mode)
    check(lib().opflow_weno_rk3_mode(u.ctx.handle, u.handle, u1.handle if u1 else None, u2.handle if u2 else None, kind, dim, float(dt),
                                     int(steps), m))


# ---------------------------------------------------------------------------------------------- batches
class Problem:
    """alpha*u - beta*Lap(u) = f on an n[0] x n[1] (x n[2]) grid of cells (Center) or nodes (Corner) with
    spacing h, Dirichlet 0 or Neumann 0 on every side (opflow_problem_desc)."""

    def __init__(self, n, h, alpha=1.0, beta=1.0, loc=LocOnMesh.Center, bc=BCType.Dirc):
        self.n, self.h, self.alpha, self.beta, self.loc, self.bc = list(n), list(h), alpha, beta, loc, bc

    def to_c(self):
        d = capi.ProblemDesc()
        d.ndim = len(self.n)
        for k in range(d.ndim):
            d.n[k] = self.n[k]
            d.h[k] = self.h[k]
        d.loc, d.bc, d.alpha, d.beta = self.loc, self.bc, float(self.alpha), float(self.beta)
        return d


def lower_equation(getter, target):
    """The C ABI's form of makeEqnSolveHandler's equation: (opflow_equation, keep-alive objects).
    `getter(e)` returns `lhs == rhs` in the unknown e; the target is leaf slot 0."""
    eq = getter(target)
    if not isinstance(eq, Equation):
        raise TypeError("the equation getter must return `lhs == rhs` (use api.Eq for a scalar lhs)")
    nodes, leaves = serialize(eq.residual_expr(), [target])
    hs = (C.c_void_p * len(leaves))(*[f.handle.value for f in leaves])
    e = capi.Equation()
    e.nodes = C.cast(nodes, C.POINTER(capi.Node))
    e.n_nodes = len(nodes)
    e.leaves = C.cast(hs, C.POINTER(C.c_void_p))
    e.n_leaves = len(leaves)
    e.unknown = 0
    return e, (nodes, hs, leaves)


class Batch:
    """Many independent problems solved together, one launch per multigrid operation for the batch.
    `problems` holds Problem descriptions, or (getter, target) pairs of user equations
    (opflow_batch_create_eqns: each assembled from its fields, started from its target's values)."""

    def __init__(self, problems, params=None, ctx=None):
        self.ctx = ctx or default_context()
        self.problems = list(problems)
        self.params = params or StructSolverParams()
        p = self.params.to_c()
        h = C.c_void_p()
        if self.problems and isinstance(self.problems[0], tuple):
            lowered = [lower_equation(g, t) for g, t in self.problems]
            self._keep = [k for _, k in lowered]
            arr = (capi.Equation * len(lowered))(*[e for e, _ in lowered])
            check(lib().opflow_batch_create_eqns(self.ctx.handle, arr, len(lowered), C.byref(p), C.byref(h)))
        else:
            arr = (capi.ProblemDesc * len(self.problems))(*[q.to_c() for q in self.problems])
            check(lib().opflow_batch_create(self.ctx.handle, arr, len(self.problems), C.byref(p), C.byref(h)))
        self.handle = h

    def size(self, i):
        n = C.c_size_t(0)
        check(lib().opflow_batch_vectors(self.handle, i, None, None, C.byref(n)))
        return n.value

    def set(self, i, f, x0=None):
        f = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        x0p = None
        if x0 is not None:
            x0 = np.ascontiguousarray(x0, dtype=np.float64).reshape(-1)
            x0p = x0.ctypes.data_as(C.POINTER(C.c_double))
        check(lib().opflow_batch_set(self.handle, i, f.ctypes.data_as(C.POINTER(C.c_double)), x0p, f.size))

    def get(self, i):
        x = np.empty(self.size(i))
        check(lib().opflow_batch_get(self.handle, i, x.ctypes.data_as(C.POINTER(C.c_double)), x.size))
        return x

    def solve(self):
        st = (capi.SolveState * len(self.problems))()
        rc = lib().opflow_batch_solve(self.handle, st)
        if rc not in (capi.OK, capi.E_NOT_CONVERGED):
            check(rc)
        return [EqnSolveState(s) for s in st]

    def close(self):
        if getattr(self, "handle", None) and not _exiting[0]:
            lib().opflow_batch_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------------------------------------ serving
def assign_batch(assignments, steps=1):
    """Many explicit assignments in one launch per step (opflow_assign_batch): `assignments` holds
    (dst, expr) or (dst, expr, op) with op one of "=", "+", "-", "*", "/" (as in CartesianField.assign),
    over fields of any sizes; the values equal
    dst.assign(expr, op, mode="exact", steps=steps) for each, step for step.  No assignment may read
    another one's destination."""
    n = len(assignments)
    if n == 0:
        return
    keep = []
    dsts, ariths, nn, nl = (C.c_void_p * n)(), (C.c_int * n)(), (C.c_int * n)(), (C.c_int * n)()
    nodes_p, leaves_p = (C.c_void_p * n)(), (C.c_void_p * n)()
    for i, a in enumerate(assignments):
        dst, expr = a[0], a[1]
        op = a[2] if len(a) > 2 else "="
        nodes, leaves = serialize(expr)
        hs = (C.c_void_p * max(1, len(leaves)))(*[f.handle.value for f in leaves])
        keep += [nodes, hs]
        dsts[i] = dst.handle.value
        ariths[i] = _ARITH[op]
        nodes_p[i] = C.cast(nodes, C.c_void_p)
        nn[i] = len(nodes)
        leaves_p[i] = C.cast(hs, C.c_void_p)
        nl[i] = len(leaves)
    check(lib().opflow_assign_batch(assignments[0][0].ctx.handle, n, dsts, ariths, nodes_p, nn, leaves_p, nl, int(steps)))


def tune_set_cache(path):
    """Autotuner cache file (opflow_tune_set_cache): choices are loaded from `path` and new ones appended;
    None keeps them in memory only."""
    check(lib().opflow_tune_set_cache(None if path is None else str(path).encode()))


def tune_lookup(key):
    """The tuned choice for `key`, or None."""
    v = C.c_int(0)
    if lib().opflow_tune_lookup(key.encode(), C.byref(v)) != capi.OK:
        return None
    return v.value


def tune_stats():
    """(choices measured by this process, cache hits, entries held)."""
    t, h, n = C.c_longlong(0), C.c_longlong(0), C.c_longlong(0)
    check(lib().opflow_tune_stats(C.byref(t), C.byref(h), C.byref(n)))
    return t.value, h.value, n.value


def tune_clear():
    check(lib().opflow_tune_clear())


class Server:
    """Request loop with continuous batching (opflow_server_*): requests of any size join the running
    batch at the next iteration boundary and leave when they converge; heat sessions (steps > 1) stay
    resident between their steps."""

    def __init__(self, params=None, hbm_budget=0, max_active=64, ctx=None):
        self.ctx = ctx or default_context()
        self.params = params or StructSolverParams(precision="mixed")
        p = self.params.to_c()
        h = C.c_void_p()
        check(lib().opflow_server_create(self.ctx.handle, C.byref(p), int(hbm_budget), int(max_active), C.byref(h)))
        self.handle = h
        self._keep = {}

    @staticmethod
    def _ptr(a):
        """Address of a float64 buffer: a numpy array (host) or any object with a CUDA device pointer
        (a contiguous float64 torch tensor on the GPU: device-resident requests)."""
        if hasattr(a, "data_ptr") and getattr(a, "is_cuda", False):
            assert a.is_contiguous() and str(a.dtype) == "torch.float64"
            return a, C.cast(C.c_void_p(a.data_ptr()), C.POINTER(C.c_double))
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        return a, a.ctypes.data_as(C.POINTER(C.c_double))

    def submit(self, problem, f, steps=1, out=None, x0=None):
        """Queues a request; x0 is the first solve's initial guess (a restored session's checkpoint).
        f, out and x0 are host arrays or device tensors (the library copies with unified addressing)."""
        f, fp = self._ptr(f)
        req = capi.Request()
        req.problem = problem.to_c()
        req.steps = int(steps)
        req.f = fp
        if x0 is not None:
            x0, req.x0 = self._ptr(x0)
        if out is not None:
            if hasattr(out, "data_ptr") and getattr(out, "is_cuda", False):
                out, req.x_out = self._ptr(out)
            else:
                assert out.dtype == np.float64 and out.flags["C_CONTIGUOUS"]
                req.x_out = out.ctypes.data_as(C.POINTER(C.c_double))
        rid = C.c_longlong(0)
        check(lib().opflow_server_submit(self.handle, C.byref(req), C.byref(rid)))
        self._keep[rid.value] = (f, out, x0)
        return rid.value

    def submit_equation(self, getter, target, out=None, x0=None):
        """Queues one solve of a user equation (`getter(e)` returns `lhs == rhs` in the unknown e, as
        for makeEqnSolveHandler): assembled from its fields at admission, so they must stay unchanged
        until the result; started from the target's values unless x0 is given; the solution over the
        target's assignable cells goes to `out` (the target itself is not written)."""
        e, keep = lower_equation(getter, target)
        req = capi.Request()
        req.steps = 1
        req.equation = C.pointer(e)
        if x0 is not None:
            x0, req.x0 = self._ptr(x0)
        if out is not None:
            if hasattr(out, "data_ptr") and getattr(out, "is_cuda", False):
                out, req.x_out = self._ptr(out)
            else:
                assert out.dtype == np.float64 and out.flags["C_CONTIGUOUS"]
                req.x_out = out.ctypes.data_as(C.POINTER(C.c_double))
        rid = C.c_longlong(0)
        check(lib().opflow_server_submit(self.handle, C.byref(req), C.byref(rid)))
        self._keep[rid.value] = (e, keep, out, x0)
        return rid.value

    def checkpoint(self, rid, n):
        """(state, steps done) of a running session at its next step boundary (opflow_server_checkpoint)."""
        x = np.empty(int(n))
        k = C.c_int(0)
        check(lib().opflow_server_checkpoint(self.handle, rid, x.ctypes.data_as(C.POINTER(C.c_double)), x.size, C.byref(k)))
        return x, k.value

    def result(self, rid, wait=True):
        res = capi.RequestResult()
        done = C.c_int(0)
        check(lib().opflow_server_result(self.handle, rid, int(wait), C.byref(done), C.byref(res)))
        if not done.value:
            return None
        self._keep.pop(rid, None)
        return {"id": res.id, "status": res.status, "iterations": res.iterations, "solves": res.solves,
                "rel_residual": res.rel_residual, "queue_ms": res.queue_ms, "latency_ms": res.latency_ms}

    def drain(self):
        check(lib().opflow_server_drain(self.handle))

    def stats(self):
        st = capi.ServeStats()
        check(lib().opflow_server_stats(self.handle, C.byref(st)))
        return {k: getattr(st, k) for k, _ in capi.ServeStats._fields_}

    def close(self):
        if getattr(self, "handle", None) and not _exiting[0]:
            lib().opflow_server_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
