"""EOM / IC string language of pyranda (pyranda/pyrandaUtils.py:22-141).

``:name:`` marks a scalar variable, ``:[name]:`` a vector; a translation map
(sMap) rewrites operator and function names into calls on the simulation
object.  The replacement order is the map's insertion order, as in the
reference.
"""
import re

scalar_key = ":"
vector_key = [":[", "]:"]
tensor_key = [":{", "}:"]


def fortran3d(form, sMap):
    """Translate one EOM/IC line into a Python expression (pyrandaUtils.py:22-66)."""
    form = form.replace(" ", "").strip()
    var_data = 'self.variables["%s"].data'
    for ivar in findVar(form, "scalar"):
        kvar = "%s%s%s" % (scalar_key, ivar, scalar_key)
        if kvar not in sMap:
            sMap[kvar] = var_data % ivar
    for ivar in findVar(form, "vector"):
        kvar = "%s%s%s" % (vector_key[0], ivar, vector_key[1])
        if kvar not in sMap:
            sMap[kvar] = var_data % ivar
    for mvar in sMap:
        if "#arg#" in mvar:
            eMap = sMap[mvar]
            prefix = mvar.split("(")[0]
            found = re.findall(re.escape(prefix) + r"\(.*?\)", form)
            if found:
                args = found[0].replace("(", "").replace(")", "").replace(prefix, "")
                form = form.replace(mvar.replace("#arg#", args), eMap.replace("#arg#", args))
        else:
            form = form.replace(mvar, sMap[mvar])
    return form


def splitLines(aLongString):
    lines = [el.replace(" ", "") for el in aLongString.split("\n") if el]
    lines = [el for el in lines if el]
    return [el for el in lines if el.strip()[0] != "#"]


def findVar(string, kind, unique=True):
    """Variable names marked in a line (pyrandaUtils.py:82-141)."""
    if kind == "scalar":
        out = _find_scalar(string)
    elif kind == "vector":
        out = _find_vecten(string, vector_key)
    elif kind == "tensor":
        out = _find_vecten(string, tensor_key)
    else:
        out = []
    if unique:
        out = list(set(out))
    return out


def _find_scalar(string):
    out = []
    for nv in re.findall("%s.*?%s" % (scalar_key, scalar_key), string):
        if not any(ch in nv for ch in "[]{}#%*@"):
            out.append(nv.replace(scalar_key, ""))
    return out


def _find_vecten(string, key):
    left, right = re.escape(key[0]), re.escape(key[1])
    return [s.replace(key[0], "").replace(key[1], "") for s in re.findall("%s.*?%s" % (left, right), string)]
