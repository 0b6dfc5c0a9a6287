"""Minimal Taichi-semantics interpreter used ONLY to generate golden fixtures.

Test infrastructure, not product code.  Taichi is not installable here, so this
module stands in for ``import taichi`` while the reference's own, unmodified
``src/simulator/simulation_functions.py`` is imported and executed in plain
Python.  It implements exactly the subset of the Taichi language that file
uses:

* fields (scalar / vector / matrix, ``ti.root.dense(...).place``, ``lazy_grad``,
  ``.grad`` companions, ``from_numpy``/``to_numpy``), struct-for iteration;
* ``ti.Vector`` / ``ti.Matrix`` arithmetic (``@``, elementwise ``*``, ``**``,
  ``transpose``, ``determinant``, ``norm``, ``norm_sqr``, ``normalized``,
  ``dot``, ``outer_product``, component call ``v(0)``);
* ``ti.atomic_add`` and ``field[idx] += v`` as atomic adds;
* ``@ti.kernel`` with a ``.grad`` reverse-mode companion, ``@ti.func``,
  ``ti.ad.Tape``, ``ti.ad.grad_replaced`` / ``ti.ad.grad_for``;
* ``ti.svd`` (3x3, numpy; its outputs are never consumed by the reference).

Reverse mode follows Taichi's documented semantics: a kernel's ``.grad`` re-reads
the primal fields as they are (it does not re-run stores), every global load is
a leaf whose adjoint is accumulated into ``field.grad``, and every global store
or atomic add seeds its value's adjoint from ``field.grad`` at that location.
Each outermost loop iteration is reversed on its own, which is equivalent to
Taichi's per-thread reversal because the reference's kernels never read, in one
iteration, a location that another iteration writes.

Arithmetic runs in float64 (``set_precision('f64')``) or with every operation
rounded to float32 (``'f32'``), selectable per fixture.
"""

import builtins
import math
import sys
import types

import numpy as np

# ----------------------------------------------------------------------------
# precision / rounding
# ----------------------------------------------------------------------------
_STATE = types.SimpleNamespace(prec='f64', ad=False, tape=None, top_active=False,
                               target_tape=None, grad_replaced=False, fields=[])


def set_precision(p):
    assert p in ('f32', 'f64')
    _STATE.prec = p


def _rnd(x):
    if _STATE.prec == 'f32':
        return float(np.float32(x))
    return float(x)


# ----------------------------------------------------------------------------
# scalar with optional reverse-mode tracking
# ----------------------------------------------------------------------------
class Var:
    __slots__ = ('v', 'parents', 'g', 'leaf', 'ref')

    def __init__(self, v, parents=None, leaf=None, ref=None):
        self.v = v
        self.parents = parents
        self.g = 0.0
        self.leaf = leaf          # (field, index_tuple, component) for loads
        self.ref = ref            # (field, index) of a direct subscript result
        if _STATE.ad and (parents or leaf is not None):
            _STATE.tape.append(self)

    # --- helpers -----------------------------------------------------------
    def __float__(self):
        return float(self.v)

    def __repr__(self):
        return 'Var(%r)' % (self.v,)

    # comparisons use values (branches are not differentiated)
    def __lt__(self, o): return self.v < _val(o)
    def __le__(self, o): return self.v <= _val(o)
    def __gt__(self, o): return self.v > _val(o)
    def __ge__(self, o): return self.v >= _val(o)
    def __eq__(self, o): return self.v == _val(o)
    def __ne__(self, o): return self.v != _val(o)
    __hash__ = object.__hash__

    def __add__(self, o): return NotImplemented if _nonscalar(o) else _add(self, o)
    def __radd__(self, o): return _add(o, self)
    def __sub__(self, o): return NotImplemented if _nonscalar(o) else _sub(self, o)
    def __rsub__(self, o): return _sub(o, self)
    def __mul__(self, o): return NotImplemented if _nonscalar(o) else _mul(self, o)
    def __rmul__(self, o): return _mul(o, self)
    def __truediv__(self, o): return NotImplemented if _nonscalar(o) else _div(self, o)
    def __rtruediv__(self, o): return _div(o, self)
    def __pow__(self, o): return NotImplemented if _nonscalar(o) else _pow(self, o)
    def __rpow__(self, o): return _pow(o, self)
    def __neg__(self): return _mul(self, -1.0)
    def __pos__(self): return self
    def __abs__(self): return _abs(self)

    def __iadd__(self, o):
        if self.ref is not None:
            fld, idx = self.ref
            fld._atomic(idx, o)
            return _ATOMIC_DONE
        return _add(self, o)


class _AtomicDone:
    pass


_ATOMIC_DONE = _AtomicDone()


def _nonscalar(o):
    return isinstance(o, (Mat, list, tuple))


def _val(a):
    if isinstance(a, Var):
        return a.v
    return a


def _mk(v, parents):
    """Create a result scalar.  ``parents`` is a list of (Var, partial)."""
    v = _rnd(v)
    if _STATE.ad:
        ps = [(p, d) for (p, d) in parents if isinstance(p, Var)]
        if ps:
            return Var(v, ps)
    if any(isinstance(p, Var) for p, _ in parents):
        return Var(v)
    return v


def _is_num(a):
    return isinstance(a, (Var, int, float, np.floating, np.integer))


def _add(a, b):
    if not isinstance(a, Var) and not isinstance(b, Var):
        if isinstance(a, int) and isinstance(b, int):
            return a + b
        return _rnd(float(a) + float(b))
    return _mk(_val(a) + _val(b), [(a, 1.0), (b, 1.0)])


def _sub(a, b):
    if not isinstance(a, Var) and not isinstance(b, Var):
        if isinstance(a, int) and isinstance(b, int):
            return a - b
        return _rnd(float(a) - float(b))
    return _mk(_val(a) - _val(b), [(a, 1.0), (b, -1.0)])


def _mul(a, b):
    if not isinstance(a, Var) and not isinstance(b, Var):
        if isinstance(a, int) and isinstance(b, int):
            return a * b
        return _rnd(float(a) * float(b))
    va, vb = _val(a), _val(b)
    return _mk(va * vb, [(a, vb), (b, va)])


def _div(a, b):
    va, vb = float(_val(a)), float(_val(b))
    if vb == 0.0:
        q = math.copysign(math.inf, va) if va != 0 else math.nan
    else:
        q = va / vb
    if not isinstance(a, Var) and not isinstance(b, Var):
        return _rnd(q)
    return _mk(q, [(a, 1.0 / vb if vb != 0 else math.inf), (b, -q / vb if vb != 0 else math.inf)])


def _pow(a, b):
    va, vb = float(_val(a)), float(_val(b))
    try:
        r = va ** vb
    except ZeroDivisionError:
        r = math.inf
    if isinstance(r, complex):
        r = math.nan
    if not isinstance(a, Var) and not isinstance(b, Var):
        if isinstance(a, int) and isinstance(b, int) and b >= 0:
            return a ** b
        return _rnd(r)
    if va == 0.0:
        da = 0.0 if vb > 1.0 else (1.0 if vb == 1.0 else math.inf)
    else:
        try:
            da = vb * (va ** (vb - 1.0))
        except (ZeroDivisionError, OverflowError):
            da = math.inf
        if isinstance(da, complex):
            da = math.nan
    db = r * math.log(va) if va > 0 else (0.0 if not isinstance(b, Var) else math.nan)
    return _mk(r, [(a, da), (b, db)])


def _abs(a):
    va = _val(a)
    if not isinstance(a, Var):
        return abs(va)
    s = 1.0 if va > 0 else (-1.0 if va < 0 else 0.0)
    return _mk(abs(va), [(a, s)])


def _sqrt(a):
    va = float(_val(a))
    r = math.sqrt(va) if va >= 0 else math.nan
    if not isinstance(a, Var):
        return _rnd(r)
    d = 0.5 / r if r > 0 else math.inf
    return _mk(r, [(a, d)])


def _backprop(tape):
    """Reverse sweep over one outermost-loop iteration's tape."""
    for node in reversed(tape):
        if isinstance(node, _Write):
            fld, idx, comp, var = node.fld, node.idx, node.comp, node.var
            seed = fld.grad._get_comp(idx, comp)
            if isinstance(var, Var) and seed != 0.0:
                var.g += seed
            continue
        g = node.g
        if g == 0.0:
            continue
        if node.leaf is not None:
            fld, idx, comp = node.leaf
            fld.grad._add_comp(idx, comp, g)
        if node.parents:
            for p, d in node.parents:
                if d == 0.0:
                    continue
                p.g += g * d


class _Write:
    __slots__ = ('fld', 'idx', 'comp', 'var')

    def __init__(self, fld, idx, comp, var):
        self.fld, self.idx, self.comp, self.var = fld, idx, comp, var


def _flush():
    if _STATE.ad and _STATE.tape:
        tape = _STATE.tape
        _STATE.tape = []
        _backprop(tape)


# ----------------------------------------------------------------------------
# small matrices / vectors
# ----------------------------------------------------------------------------
def _conv(e):
    if isinstance(e, (Var, int)):
        return e
    if isinstance(e, (np.integer,)):
        return int(e)
    return _rnd(float(e))


class Mat:
    """Row-major n x m matrix of scalars; ``vec`` marks a column vector."""
    __slots__ = ('n', 'm', 'e', 'vec', 'ref')

    def __init__(self, rows, vec=False, dt=None):
        if vec:
            self.e = [[_conv(x)] for x in rows]
            self.n, self.m = len(rows), 1
        else:
            self.e = [[_conv(x) for x in r] for r in rows]
            self.n, self.m = len(rows), len(rows[0])
        self.vec = vec
        self.ref = None

    # construction helpers --------------------------------------------------
    @staticmethod
    def _from(e, vec):
        o = Mat.__new__(Mat)
        o.e = e
        o.n, o.m = len(e), len(e[0])
        o.vec = vec
        o.ref = None
        return o

    def _map2(self, o, fn):
        if isinstance(o, Mat):
            assert o.n == self.n and o.m == self.m, 'shape mismatch'
            return Mat._from([[fn(self.e[i][j], o.e[i][j]) for j in range(self.m)]
                              for i in range(self.n)], self.vec)
        if isinstance(o, (list, tuple)):
            return self._map2(Mat(list(o), vec=True) if self.vec else Mat(o), fn)
        return Mat._from([[fn(self.e[i][j], o) for j in range(self.m)]
                          for i in range(self.n)], self.vec)

    def _rmap2(self, o, fn):
        if isinstance(o, (list, tuple)):
            return (Mat(list(o), vec=True) if self.vec else Mat(o))._map2(self, fn)
        return Mat._from([[fn(o, self.e[i][j]) for j in range(self.m)]
                          for i in range(self.n)], self.vec)

    def __add__(self, o): return self._map2(o, _add)
    def __radd__(self, o): return self._rmap2(o, _add)
    def __sub__(self, o): return self._map2(o, _sub)
    def __rsub__(self, o): return self._rmap2(o, _sub)
    def __mul__(self, o): return self._map2(o, _mul)
    def __rmul__(self, o): return self._rmap2(o, _mul)
    def __truediv__(self, o): return self._map2(o, _div)
    def __rtruediv__(self, o): return self._rmap2(o, _div)
    def __pow__(self, o): return self._map2(o, _pow)
    def __neg__(self): return self._map2(-1.0, _mul)

    def __iadd__(self, o):
        if self.ref is not None:
            fld, idx = self.ref
            fld._atomic(idx, o)
            return _ATOMIC_DONE
        return self.__add__(o)

    def __isub__(self, o):
        return self.__sub__(o)

    def __matmul__(self, o):
        assert isinstance(o, Mat) and self.m == o.n
        out = []
        for i in range(self.n):
            row = []
            for j in range(o.m):
                acc = _mul(self.e[i][0], o.e[0][j])
                for k in range(1, self.m):
                    acc = _add(acc, _mul(self.e[i][k], o.e[k][j]))
                row.append(acc)
            out.append(row)
        return Mat._from(out, o.vec)

    def __getitem__(self, k):
        if isinstance(k, tuple):
            return self.e[k[0]][k[1]]
        if self.vec or self.m == 1:
            return self.e[k][0]
        return Mat._from([[x] for x in self.e[k]], True)

    def __setitem__(self, k, v):
        if isinstance(k, tuple):
            self.e[k[0]][k[1]] = _conv(v)
        else:
            self.e[k][0] = _conv(v)

    def __call__(self, *k):
        if len(k) == 1:
            return self[k[0]]
        return self.e[k[0]][k[1]]

    def __iter__(self):
        if self.vec:
            return iter([r[0] for r in self.e])
        return iter([Mat._from([[x] for x in r], True) for r in self.e])

    def transpose(self):
        return Mat._from([[self.e[i][j] for i in range(self.n)] for j in range(self.m)], False)

    def determinant(self):
        a = self.e
        assert self.n == 3 and self.m == 3
        t0 = _sub(_mul(a[1][1], a[2][2]), _mul(a[1][2], a[2][1]))
        t1 = _sub(_mul(a[1][0], a[2][2]), _mul(a[1][2], a[2][0]))
        t2 = _sub(_mul(a[1][0], a[2][1]), _mul(a[1][1], a[2][0]))
        return _add(_sub(_mul(a[0][0], t0), _mul(a[0][1], t1)), _mul(a[0][2], t2))

    def norm_sqr(self):
        acc = None
        for r in self.e:
            for x in r:
                t = _mul(x, x)
                acc = t if acc is None else _add(acc, t)
        return acc

    def norm(self, eps=0):
        s = self.norm_sqr()
        if eps:
            s = _add(s, eps)
        return _sqrt(s)

    def normalized(self, eps=0):
        return self * _div(1.0, self.norm(eps))

    def dot(self, o):
        acc = None
        for i in range(self.n):
            t = _mul(self.e[i][0], o.e[i][0])
            acc = t if acc is None else _add(acc, t)
        return acc

    def outer_product(self, o):
        return Mat._from([[_mul(self.e[i][0], o.e[j][0]) for j in range(o.n)]
                          for i in range(self.n)], False)

    def values(self):
        return [[float(_val(x)) for x in r] for r in self.e]


def _as_components(value, n, m):
    """Flatten a value to a list of n*m components (row-major)."""
    if isinstance(value, Mat):
        return [value.e[i][j] for i in range(value.n) for j in range(value.m)]
    if isinstance(value, (list, tuple)):
        out = []
        for r in value:
            if isinstance(r, (list, tuple)):
                out.extend(_conv(x) for x in r)
            else:
                out.append(_conv(r))
        return out
    return [_conv(value)]


# ----------------------------------------------------------------------------
# fields
# ----------------------------------------------------------------------------
class Field:
    def __init__(self, n=None, m=None, dtype='f32', shape=None, is_grad=False):
        self.n, self.m = n, m          # None/None scalar, n/None vector, n/m matrix
        self.dtype = dtype
        self.shape = None
        self.data = None
        self.grad = None
        self.is_grad = is_grad
        if shape is not None:
            self._alloc(shape if isinstance(shape, tuple) else (shape,))
        if not is_grad:
            _STATE.fields.append(self)

    @property
    def ncomp(self):
        if self.n is None:
            return 1
        return self.n * (self.m or 1)

    def _alloc(self, shape):
        self.shape = tuple(shape)
        np_dt = np.int64 if self.dtype == 'i32' else np.float64
        self.data = np.zeros(self.shape + (self.ncomp,), dtype=np_dt)
        if self.dtype != 'i32' and not self.is_grad:
            self.grad = Field(self.n, self.m, self.dtype, None, is_grad=True)
            self.grad._alloc(self.shape)

    # index normalisation -------------------------------------------------
    def _idx(self, k):
        if k is None:
            return ()
        if isinstance(k, Mat):
            return tuple(int(_val(x)) for x in k)
        if isinstance(k, tuple):
            return tuple(int(_val(x)) for x in k)
        return (int(_val(k)),)

    def _get_comp(self, idx, c):
        return float(self.data[idx + (c,)])

    def _add_comp(self, idx, c, g):
        self.data[idx + (c,)] += g

    def __getitem__(self, k):
        idx = self._idx(k)
        row = self.data[idx]
        if self.dtype == 'i32':
            if self.n is None:
                return int(row[0])
            vals = [int(x) for x in row]
        else:
            if _STATE.ad and not self.is_grad:
                vals = [Var(float(row[c]), leaf=(self, idx, c)) for c in range(self.ncomp)]
            else:
                vals = [float(row[c]) for c in range(self.ncomp)]
            if self.n is None:
                v = vals[0]
                if not isinstance(v, Var):
                    v = Var(v)
                v.ref = (self, idx)
                return v
        if self.n is None:
            return vals[0]
        if self.m is None:
            out = Mat(vals, vec=True)
        else:
            out = Mat([vals[i * self.m:(i + 1) * self.m] for i in range(self.n)])
        out.ref = (self, idx)
        return out

    def __setitem__(self, k, value):
        if value is _ATOMIC_DONE:
            return
        idx = self._idx(k)
        comps = _as_components(value, self.n or 1, self.m or 1)
        if len(comps) == 1 and self.ncomp > 1:
            comps = comps * self.ncomp
        if _STATE.ad and not self.is_grad:
            for c, x in enumerate(comps):
                _STATE.tape.append(_Write(self, idx, c, x))
            return
        for c, x in enumerate(comps):
            self.data[idx + (c,)] = _rnd(_val(x)) if self.dtype != 'i32' else int(_val(x))

    def _atomic(self, idx, value):
        comps = _as_components(value, self.n or 1, self.m or 1)
        if _STATE.ad and not self.is_grad:
            for c, x in enumerate(comps):
                _STATE.tape.append(_Write(self, idx, c, x))
            return
        for c, x in enumerate(comps):
            self.data[idx + (c,)] = _rnd(self.data[idx + (c,)] + _val(x))

    def __iter__(self):
        return _TopIter(np.ndindex(*self.shape))

    # python-scope API ------------------------------------------------------
    def from_numpy(self, arr):
        arr = np.asarray(arr)
        want = self.shape + ((self.n,) if self.n else ()) + ((self.m,) if self.m else ())
        assert arr.shape == want, 'from_numpy shape %s != field shape %s' % (arr.shape, want)
        flat = arr.reshape(self.shape + (self.ncomp,))
        if self.dtype == 'i32':
            self.data[...] = flat.astype(np.int64)
        else:
            self.data[...] = np.vectorize(_rnd)(flat.astype(np.float64)) if _STATE.prec == 'f32' else flat

    def to_numpy(self):
        want = self.shape + ((self.n,) if self.n else ()) + ((self.m,) if self.m else ())
        return self.data.reshape(want).copy()

    def fill(self, v):
        self.data[...] = v


class _TopIter:
    """Iterator for kernel-level loops: reverses the tape once per iteration."""

    def __init__(self, it):
        self.it = iter(it)
        self.top = None

    def __iter__(self):
        return self

    def __next__(self):
        if self.top is None:
            self.top = not _STATE.top_active
            if self.top:
                _STATE.top_active = True
        if self.top:
            _flush()
        try:
            return next(self.it)
        except StopIteration:
            if self.top:
                _STATE.top_active = False
            raise


def shim_range(*a):
    return _TopIter(builtins.range(*a))


# ----------------------------------------------------------------------------
# layout builders (ti.root.dense(...).place)
# ----------------------------------------------------------------------------
class _SNode:
    def __init__(self, shape=()):
        self.shape = shape

    def dense(self, axes, n):
        if isinstance(n, (tuple, list)):
            return _SNode(self.shape + tuple(n))
        if isinstance(axes, tuple) and len(axes) > 1:
            return _SNode(self.shape + (n,) * len(axes))
        return _SNode(self.shape + (n,))

    def place(self, *fields):
        for f in fields:
            f._alloc(self.shape)
        return self

    def lazy_grad(self):
        pass


root = _SNode(())
i = ('i',)
j = ('j',)
k = ('k',)
l = ('l',)
ij = ('i', 'j')
ijk = ('i', 'j', 'k')
i32 = 'i32'
f32 = 'f32'
f64 = 'f64'
cuda = 'cuda'
cpu = 'cpu'


def field(dtype=f32, shape=None, needs_grad=False):
    return Field(None, None, dtype, shape)


def init(*a, **kw):
    pass


def reset():
    pass


def static(x, *a):
    return x


def ndrange(*dims):
    import itertools
    return list(itertools.product(*[builtins.range(d) for d in dims]))


def cast(x, dtype):
    if dtype == i32 or dtype is int:
        if isinstance(x, Mat):
            return Mat._from([[int(math.trunc(_val(e))) for e in r] for r in x.e], x.vec)
        return int(math.trunc(_val(x)))
    if isinstance(x, Mat):
        return Mat._from([[_conv(float(e)) if not isinstance(e, Var) else e for e in r] for r in x.e], x.vec)
    return _conv(float(x)) if not isinstance(x, Var) else x


def atomic_add(dst, value):
    ref = getattr(dst, 'ref', None)
    assert ref is not None, 'atomic_add target must be a field subscript'
    fld, idx = ref
    fld._atomic(idx, value)


def sqrt(x):
    return _sqrt(x)


def max(a, b):
    return a if _val(a) >= _val(b) else b


def min(a, b):
    return a if _val(a) <= _val(b) else b


def func(fn):
    return fn


def svd(A, dt=None):
    a = np.array(A.values(), dtype=np.float64)
    U, s, Vt = np.linalg.svd(a)
    V = Vt.T
    if np.linalg.det(U) < 0:
        U[:, 2] *= -1
        s[2] *= -1
    if np.linalg.det(V) < 0:
        V[:, 2] *= -1
        s[2] *= -1
    S = np.diag(s)
    return Mat(U.tolist()), Mat(S.tolist()), Mat(V.tolist())


class _VectorNS:
    def __call__(self, vals, dt=None):
        return Mat(list(vals), vec=True)

    @staticmethod
    def field(n, dtype=f32, shape=None, needs_grad=False):
        return Field(n, None, dtype, shape)

    @staticmethod
    def zero(dtype, n):
        return Mat([0.0] * n, vec=True)


class _MatrixNS:
    def __call__(self, rows, dt=None):
        return Mat(rows)

    @staticmethod
    def field(n, m, dtype=f32, shape=None, needs_grad=False):
        return Field(n, m, dtype, shape)

    @staticmethod
    def zero(dtype, n, m):
        return Mat([[0.0] * m for _ in builtins.range(n)])

    @staticmethod
    def identity(dtype, n):
        return Mat([[1.0 if a == b else 0.0 for b in builtins.range(n)] for a in builtins.range(n)])


Vector = _VectorNS()
Matrix = _MatrixNS()


# ----------------------------------------------------------------------------
# kernels, tape
# ----------------------------------------------------------------------------
class Kernel:
    def __init__(self, fn):
        self.fn = fn
        self.__name__ = fn.__name__
        self.grad = _GradKernel(self)

    def __call__(self, *args):
        tape = _STATE.target_tape
        if tape is not None and not _STATE.grad_replaced and not tape.replaying:
            tape.calls.append((self, args))
        prev = (_STATE.ad, _STATE.top_active)
        _STATE.ad, _STATE.top_active = False, False
        try:
            return self.fn(*args)
        finally:
            _STATE.ad, _STATE.top_active = prev


class _GradKernel:
    def __init__(self, k):
        self.k = k

    def __call__(self, *args):
        prev = (_STATE.ad, _STATE.tape, _STATE.top_active)
        _STATE.ad, _STATE.tape, _STATE.top_active = True, [], False
        try:
            self.k.fn(*args)
            _flush()
        finally:
            _STATE.ad, _STATE.tape, _STATE.top_active = prev


def kernel(fn):
    return Kernel(fn)


def clear_all_gradients():
    for f in _STATE.fields:
        if f.grad is not None and f.grad.data is not None:
            f.grad.data[...] = 0.0


class Tape:
    def __init__(self, loss=None, clear_gradients=True):
        self.loss = loss
        self.clear = clear_gradients
        self.calls = []
        self.replaying = False

    def __enter__(self):
        if self.clear:
            clear_all_gradients()
        _STATE.target_tape = self
        return self

    def __exit__(self, *exc):
        _STATE.target_tape = None
        if exc[0] is not None:
            return False
        self.replaying = True
        self.loss.grad.data[...] = 1.0
        for fn, args in reversed(self.calls):
            fn.grad(*args)
        self.replaying = False
        return False


class _GradReplaced:
    def __init__(self, fn):
        self.fn = fn
        self.grad = None

    def __call__(self, *args):
        tape = _STATE.target_tape
        if tape is not None and not tape.replaying:
            tape.calls.append((self, args))
        _STATE.grad_replaced = True
        try:
            return self.fn(*args)
        finally:
            _STATE.grad_replaced = False


def _grad_replaced(fn):
    return _GradReplaced(fn)


def _grad_for(primal):
    def deco(fn):
        primal.grad = fn
        return fn
    return deco


ad = types.SimpleNamespace(Tape=Tape, grad_replaced=_grad_replaced, grad_for=_grad_for,
                           clear_all_gradients=clear_all_gradients)


def install():
    """Register this module as ``taichi`` and stub the visualisation imports."""
    mod = sys.modules[__name__]
    sys.modules['taichi'] = mod
    for name in ('open3d', 'matplotlib', 'matplotlib.pyplot'):
        if name not in sys.modules:
            stub = types.ModuleType(name)
            sys.modules[name] = stub
    sys.modules['matplotlib'].pyplot = sys.modules['matplotlib.pyplot']
    return mod
