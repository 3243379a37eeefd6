"""OpenFOAM dictionaries and FoamAdapter's fvSolution / fvSchemes mapping.

Python mirror of the host side that FoamAdapter builds on OpenFOAM:

* ``Dictionary`` is NeoN::Dictionary as FoamAdapter::convert fills it from a
  Foam::dictionary (src/auxiliary/foamDictionary.cpp:12-91): ``get`` gives a
  label (int) for a single integer token, a scalar (float) for a single
  floating-point token, a Vec3 (3-tuple of floats) for ``(x y z)``, a word
  (str) for a single word or quoted string, else the token list (list of int,
  float and str), and a ``Dictionary`` for a sub-dictionary;
* ``update_solver``, ``update_preconditioner``, ``update_criteria`` and
  ``map_fv_solution`` are FoamAdapter::updateSolver / updatePreconditioner /
  updateCriteria / mapFvSolution (src/compatibility/fvSolution.cpp:19-159);
* ``solver_config`` turns a mapped solver entry into the keyword arguments of
  ``neon.LinearSystem.solve``; ``scheme`` reads fvSchemes.

Parsing and mapping run in libfvgb (``csrc/foamdict.cpp``, ``fvgb_dict_*``);
this module holds handles to its dictionaries.
"""
from __future__ import annotations

import ctypes as C
import re

from . import abi

_WORD = re.compile(r"^[A-Za-z_][^\s;{}()\[\]\"]*$")


class Dictionary:
    """A dictionary of libfvgb (``fvgb_dict``).  A sub-dictionary returned by
    ``subDict`` or ``get`` is a view that stays valid until its entry is
    replaced or removed (as a reference from NeoN::Dictionary::subDict)."""

    def __init__(self, handle, owner: "Dictionary | None" = None):
        if not handle:
            raise ValueError("null dictionary handle")
        self.handle = handle
        self._owner = owner  # the top-level dictionary this view belongs to

    # ---------------------------------------------------------- construction
    @classmethod
    def read(cls, path) -> "Dictionary":
        h = C.c_void_p()
        abi.check(abi.lib().fvgb_dict_read(str(path).encode(), C.byref(h)))
        return cls(h.value)

    @classmethod
    def parse(cls, text: str, include_dir=None) -> "Dictionary":
        h = C.c_void_p()
        inc = None if include_dir is None else str(include_dir).encode()
        abi.check(abi.lib().fvgb_dict_parse(text.encode(), inc, C.byref(h)))
        return cls(h.value)

    @classmethod
    def empty(cls) -> "Dictionary":
        h = C.c_void_p()
        abi.check(abi.lib().fvgb_dict_create(C.byref(h)))
        return cls(h.value)

    def copy(self) -> "Dictionary":
        h = C.c_void_p()
        abi.check(abi.lib().fvgb_dict_copy(self.handle, C.byref(h)))
        return Dictionary(h.value)

    def close(self):
        if self.handle and self._owner is None:
            abi.lib().fvgb_dict_free(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --------------------------------------------------------------- queries
    def _index(self, key: str) -> int:
        return abi.lib().fvgb_dict_find(self.handle, key.encode())

    def _at(self, key: str) -> int:
        i = self._index(key)
        if i < 0:
            raise KeyError(key)
        return i

    def keys(self) -> list[str]:
        L = abi.lib()
        return [L.fvgb_dict_key(self.handle, i).decode() for i in range(L.fvgb_dict_size(self.handle))]

    def contains(self, key: str) -> bool:
        return self._index(key) >= 0

    __contains__ = contains

    def isDict(self, key: str) -> bool:
        return bool(abi.lib().fvgb_dict_sub(self.handle, self._at(key)))

    def subDict(self, key: str) -> "Dictionary":
        sub = abi.lib().fvgb_dict_sub(self.handle, self._at(key))
        if not sub:
            raise TypeError(f"{key} is not a sub-dictionary")
        return Dictionary(sub, owner=self._owner or self)

    def raw_tokens(self, key: str) -> list[tuple[int, str, int, float]]:
        """(kind, text, label, scalar) of each token of a primitive entry."""
        L = abi.lib()
        i = self._at(key)
        n = L.fvgb_dict_ntokens(self.handle, i)
        if n < 0:
            raise TypeError(f"{key} is a sub-dictionary")
        out = []
        kind, text, lab, sca = C.c_int32(), C.c_char_p(), C.c_int64(), C.c_double()
        for j in range(n):
            abi.check(L.fvgb_dict_token(self.handle, i, j, C.byref(kind), C.byref(text), C.byref(lab), C.byref(sca)))
            out.append((kind.value, text.value.decode(), lab.value, sca.value))
        return out

    def tokens(self, key: str) -> list:
        """The entry as NeoN::TokenList: labels as int, scalars as float, words
        and strings as str (list parentheses kept as "(" and ")")."""
        return [_value(t) for t in self.raw_tokens(key)]

    def get(self, key: str):
        if self.isDict(key):
            return self.subDict(key)
        toks = self.raw_tokens(key)
        if len(toks) == 1:
            return _value(toks[0])
        if (len(toks) == 5 and toks[0][1] == "(" and toks[4][1] == ")"
                and all(t[0] in (abi.TOK_LABEL, abi.TOK_SCALAR) for t in toks[1:4])):
            return tuple(float(t[3]) for t in toks[1:4])
        return [_value(t) for t in toks]

    def get_bool(self, key: str) -> bool:
        w = self.get(key)
        if isinstance(w, str) and w in ("yes", "on", "true"):
            return True
        if isinstance(w, str) and w in ("no", "off", "false", "none"):
            return False
        raise TypeError(f"{key} = {w!r} is not a switch")

    # ------------------------------------------------------------- mutation
    def insert(self, key: str, value):
        L = abi.lib()
        if isinstance(value, Dictionary):
            abi.check(L.fvgb_dict_set_dict(self.handle, key.encode(), value.handle, None))
            return
        abi.check(L.fvgb_dict_set(self.handle, key.encode(), _text(value).encode()))

    def insert_dict(self, key: str) -> "Dictionary":
        """Insert (or replace by) an empty sub-dictionary and return it."""
        sub = C.c_void_p()
        abi.check(abi.lib().fvgb_dict_set_dict(self.handle, key.encode(), None, C.byref(sub)))
        return Dictionary(sub.value, owner=self._owner or self)

    def remove(self, key: str):
        abi.check(abi.lib().fvgb_dict_remove(self.handle, key.encode()))

    def text(self) -> str:
        n = C.c_int64()
        abi.check(abi.lib().fvgb_dict_write(self.handle, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value + 1)
        abi.check(abi.lib().fvgb_dict_write(self.handle, buf, n.value + 1, C.byref(n)))
        return buf.value.decode()

    def __repr__(self):
        return f"Dictionary({self.keys()})"


def _value(t):
    kind, text, lab, sca = t
    if kind == abi.TOK_LABEL:
        return int(lab)
    if kind == abi.TOK_SCALAR:
        return float(sca)
    return text


def _text(v) -> str:
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, int):
        return str(v)
    if isinstance(v, float):
        return repr(v)
    if isinstance(v, str):
        return v if _WORD.match(v) else '"' + v.replace('"', '\\"') + '"'
    if isinstance(v, (tuple, list)):
        return "(" + " ".join(_text(x) for x in v) + ")"
    raise TypeError(f"cannot store {type(v).__name__} in a dictionary")


def read_foam_dictionary(path) -> Dictionary:
    """FoamAdapter::convert of an IOdictionary read from `path`."""
    return Dictionary.read(path)


# ------------------------------------------------ fvSolution.cpp:19-159
def update_solver(solver_dict: Dictionary):
    abi.check(abi.lib().fvgb_fvsolution_update_solver(solver_dict.handle))


def update_preconditioner(solver_dict: Dictionary):
    abi.check(abi.lib().fvgb_fvsolution_update_preconditioner(solver_dict.handle))


def update_criteria(solver_dict: Dictionary):
    abi.check(abi.lib().fvgb_fvsolution_update_criteria(solver_dict.handle))


def map_fv_solution(solver_dict: Dictionary) -> Dictionary:
    """mapFvSolution: a mapped copy (a plain copy when configFile is given)."""
    h = C.c_void_p()
    abi.check(abi.lib().fvgb_fvsolution_map(solver_dict.handle, C.byref(h)))
    return Dictionary(h.value)


def solver_config(mapped: Dictionary, config_dir=None) -> dict:
    """Keyword arguments of ``neon.LinearSystem.solve`` for a Ginkgo-form
    solver entry (``map_fv_solution`` output, or written that way).  An entry
    naming a ``configFile`` (a Ginkgo JSON configuration) reads that file,
    relative to ``config_dir`` (the case's system directory)."""
    cfg = abi.SolverCfg()
    if mapped.contains("configFile"):
        if config_dir is None:
            raise ValueError("solver_config: the entry names a configFile; give config_dir")
        from pathlib import Path

        path = Path(config_dir) / str(mapped.get("configFile"))
        abi.check(abi.lib().fvgb_solver_cfg_from_json(str(path).encode(), C.byref(cfg)))
    else:
        abi.check(abi.lib().fvgb_solver_cfg_from_dict(mapped.handle, C.byref(cfg)))
    return _kwargs(cfg)


def ginkgo_config(path) -> dict:
    """Keyword arguments of ``neon.LinearSystem.solve`` for a Ginkgo JSON configuration file."""
    cfg = abi.SolverCfg()
    abi.check(abi.lib().fvgb_solver_cfg_from_json(str(path).encode(), C.byref(cfg)))
    return _kwargs(cfg)


def _kwargs(cfg) -> dict:
    return dict(rel_tol=cfg.rel_tol, abs_tol=cfg.abs_tol, max_iter=cfg.max_iter, precision=cfg.precision,
                inner_rel_tol=cfg.inner_rel_tol, inner_max_iter=cfg.inner_max_iter, max_outer=cfg.max_outer,
                method=cfg.method, preconditioner=cfg.preconditioner, flags=cfg.flags)


def scheme(fv_schemes: Dictionary, section: str, name: str) -> int:
    """The scheme constant (abi.SCHEME_*) fvSchemes gives `name` in `section`."""
    out = C.c_int32()
    abi.check(abi.lib().fvgb_scheme_from_dict(fv_schemes.handle, section.encode(), name.encode(), C.byref(out)))
    return out.value
