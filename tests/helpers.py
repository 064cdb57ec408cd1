"""Builders shared by the tests: a problem -> (descriptor, initial state)."""
import numpy as np

import p2de
from p2de import problems
from p2de import solver as S


def setup(problem, **kw):
    """Returns (param, md, bc, desc, U0) for a problem factory of p2de.problems."""
    out = problem(**kw)
    param, ic, bcf = out[0], out[1], out[2]
    md = S.mesh_for(param)
    bc = bcf(param, md)
    desc = S.make_descriptor(param, md, bc)
    U0 = S.evaluate_initial_condition(param, md, ic)
    return param, md, bc, desc, U0


def fields_of(obj, fields, nstage=1):
    return {f: obj.get_field(f, nstage) for f in fields}
