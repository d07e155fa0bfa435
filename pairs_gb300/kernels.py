"""Recognition of user kernels passed to Simulation.compute() / setup().

The reference turns a user's Python function into IR by walking its AST
(src/pairs/mapping/funcs.py:39-282) and prints a C/CUDA kernel from it.  This
package has no code generator: each supported kernel family is a hand-written
CUDA kernel, and compute() recognises which family a user function is by
matching its AST against a template.  A template is ordinary Python source in
which

  I, J      stand for the function's parameters (particle i, partner j),
  P_<name>  stands for a particle / feature / contact property (bound to the
            user's name, consistently, one user name per placeholder),
  S_<name>  stands for a symbol from compute(..., symbols={...}),
  L_<name>  stands for a local variable of the function,

and every other name (the reference DSL keywords: apply, delta,
squared_distance, ...), operator, constant and the statement order must be
identical.  A match therefore means the user function computes exactly the
arithmetic the CUDA kernel implements.  Anything else raises
NotImplementedError naming the function.
"""
import ast
import inspect
import textwrap

_IGNORED = {"lineno", "col_offset", "end_lineno", "end_col_offset", "ctx", "type_comment", "kind"}


class Match:
    def __init__(self, family, bindings, params):
        self.family = family
        self.bindings = bindings      # placeholder -> user name
        self.params = params

    def prop(self, placeholder):
        return self.bindings["P_" + placeholder]

    def symbol(self, placeholder):
        return self.bindings["S_" + placeholder]

    def __repr__(self):
        return f"Match({self.family}, {self.bindings})"


def _func_ast(src):
    tree = ast.parse(textwrap.dedent(src))
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef))
    return fn


class _Matcher:
    def __init__(self, params_t, params_u):
        self.bind = {}
        self.rev = {}
        for t, u in zip(params_t, params_u):
            self.bind[t] = u
            self.rev[u] = t

    def name(self, t, u):
        if t in ("I", "J") or t[:2] in ("P_", "S_", "L_"):
            if t in self.bind:
                return self.bind[t] == u
            if u in self.rev:
                return False
            self.bind[t] = u
            self.rev[u] = t
            return True
        return t == u

    def node(self, t, u):
        if type(t) is not type(u):
            return False
        if isinstance(t, ast.Name):
            return self.name(t.id, u.id)
        if isinstance(t, ast.Constant):
            num = (int, float)
            if type(t.value) in num and type(u.value) in num:
                return float(t.value) == float(u.value)
            return t.value == u.value
        if isinstance(t, ast.arg):
            return True
        for field in t._fields:
            if field in _IGNORED:
                continue
            a, b = getattr(t, field, None), getattr(u, field, None)
            if isinstance(a, list):
                if not isinstance(b, list) or len(a) != len(b):
                    return False
                if not all(self.node(x, y) if isinstance(x, ast.AST) else x == y for x, y in zip(a, b)):
                    return False
            elif isinstance(a, ast.AST):
                if not isinstance(b, ast.AST) or not self.node(a, b):
                    return False
            elif a != b and field not in ("name",):
                return False
        return True


def match(template_src, user_fn_or_src):
    """Bindings if the user function has the template's AST, else None."""
    t = _func_ast(template_src)
    src = user_fn_or_src if isinstance(user_fn_or_src, str) else inspect.getsource(user_fn_or_src)
    u = _func_ast(src)
    pt = [a.arg for a in t.args.args]
    pu = [a.arg for a in u.args.args]
    if len(pt) != len(pu):
        return None
    m = _Matcher(pt, pu)
    if len(t.body) != len(u.body):
        return None
    for a, b in zip(t.body, u.body):
        if not m.node(a, b):
            return None
    return dict(m.bind)


# ---------------------------------------------------------------------------- templates
# LJ pair force, examples/md.py:5-8
LJ_PAIR = """
def f(I, J):
    L_sr2 = 1.0 / squared_distance(I, J)
    L_sr6 = L_sr2 * L_sr2 * L_sr2 * P_sigma6[I, J]
    apply(P_force, delta(I, J) * (48.0 * L_sr6 * (L_sr6 - 0.5) * L_sr2 * P_epsilon[I, J]))
"""

# velocity-Verlet halves, examples/md.py:11-17
VV_INITIAL = """
def f(I):
    P_velocity[I] += (S_dt * 0.5) * P_force[I] / P_mass[I]
    P_position[I] += S_dt * P_velocity[I]
"""

VV_FINAL = """
def f(I):
    P_velocity[I] += (S_dt * 0.5) * P_force[I] / P_mass[I]
"""

TEMPLATES = {
    "lj_pair": LJ_PAIR,
    "vv_initial": VV_INITIAL,
    "vv_final": VV_FINAL,
}


def register(name, src):
    """Add a kernel family template (used by the DEM path)."""
    TEMPLATES[name] = src


def recognize(fn, families=None):
    """Return Match(family, bindings) for the first template the function matches."""
    src = inspect.getsource(fn) if not isinstance(fn, str) else fn
    for fam, tsrc in TEMPLATES.items():
        if families is not None and fam not in families:
            continue
        b = match(tsrc, src)
        if b is not None:
            params = [a.arg for a in _func_ast(src).args.args]
            return Match(fam, b, params)
    name = getattr(fn, "__name__", "<source>")
    raise NotImplementedError(
        f"compute(): function {name!r} is not one of the kernel families this GB300 build implements "
        f"({', '.join(sorted(TEMPLATES))}); the reference would generate code for it, this build has "
        "hand-written CUDA kernels only")
