"""Loading the committed golden fixtures (tests/golden/*.json)."""
import json
import os

import uxxxxxxxxh_gb300 as uhs

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(HERE, name)) as f:
        return json.load(f)


def reference_stencil(case: str, kind: str = "sw") -> uhs.Stencil:
    rec = load("reference_stencils.json")[case][kind]
    return uhs.Stencil(name=rec["name"], rank=rec["rank"], sizes=tuple(rec["sizes"]), lb=tuple(rec["lb"]),
                       ub=tuple(rec["ub"]), terms=[tuple(t) for t in rec["terms"]], iterations=rec["iterations"],
                       exact_order=rec["exact_order"])


def resized(st: uhs.Stencil, interior, iterations=None) -> uhs.Stencil:
    """The same expression on a grid with another interior (same halo width)."""
    rank = st.rank
    halo = [st.lb[i] for i in range(3)]
    inner = [1] * (3 - rank) + list(interior)
    sizes = tuple(n + 2 * h if i >= 3 - rank else 1 for i, (n, h) in enumerate(zip(inner, halo)))
    lb = tuple(halo)
    ub = tuple(h + n if i >= 3 - rank else 1 for i, (n, h) in enumerate(zip(inner, halo)))
    return st.with_(sizes=sizes, lb=lb, ub=ub, iterations=st.iterations if iterations is None else iterations)
