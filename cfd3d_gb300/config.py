"""Reader/writer of the reference's positional input.inp.

`read_input` follows `t_config%construct` (src/config_module.f90:100-119): 13 pairs of a
label line followed by a value line, read list-directed in this order

  name | iread rstnum | nsteady npmax ntmax bond dt_phy | nexport nprt | iturb ides |
  nscheme nmuscl nlim | timemethod local prec cfl | fluid ngas | ncav c_v c_c |
  gravity csf | rotation rpm | pref uref aoa aos tref y1ref y2ref |
  l_chord l_character scale l_domain

and returns the dict `cfd3d_gb300.abi.config_from_dict` accepts.  A restart request
(iread), which the caller serves through `Solver.solve(restart=...)`, is returned as an
option the engine itself does not take.
"""

FIELDS = [
    ["name"],
    ["iread", "rstnum"],
    ["nsteady", "npmax", "ntmax", "bond", "dt_phy"],
    ["nexport", "nprint"],
    ["iturb", "ides"],
    ["nscheme", "nmuscl", "nlim"],
    ["timemethod", "local", "prec", "cfl"],
    ["fluid", "ngas"],
    ["ncav", "c_v", "c_c"],
    ["gravity", "csf"],
    ["rotation", "rpm"],
    ["pref", "uref", "aoa", "aos", "tref", "y1ref", "y2ref"],
    ["l_chord", "l_character", "scale", "l_domain"],
]
REALS = {"dt_phy", "cfl", "c_v", "c_c", "rpm", "pref", "uref", "aoa", "aos", "tref", "y1ref", "y2ref",
         "l_chord", "l_character", "scale", "l_domain"}
UNSUPPORTED = {"iread": 0}


def _num(tok, real):
    t = tok.strip().lower().replace("d", "e")
    return float(t) if real else int(float(t))


def read_input(text):
    """Parse the text of an input.inp; returns (config dict, list of unsupported options)."""
    lines = [l for l in text.splitlines()]
    out = {}
    pos = 0
    for group in FIELDS:
        pos += 1  # label line
        vals = lines[pos].replace(",", " ").split()
        pos += 1
        for name, tok in zip(group, vals):
            out[name] = tok if name == "name" else _num(tok, name in REALS)
    bad = [k for k, v in UNSUPPORTED.items() if out.get(k, v) != v]
    return out, bad


def write_input(cfg, name="case"):
    """Inverse of read_input (labels as in bin/input_templet.inp)."""
    d = dict(cfg)
    d.setdefault("name", name)
    for k in ("iread", "rstnum", "nexport", "nprint", "gravity", "csf", "rotation"):
        d.setdefault(k, 0)
    d.setdefault("rpm", 0.0)
    rows = []
    for group in FIELDS:
        rows.append("  ".join(group))
        vals = []
        for k in group:
            v = d.get(k, 0)
            vals.append(repr(float(v)).replace("e", "d") if k in REALS else str(v))
        rows.append("  ".join(vals))
    return "\n".join(rows) + "\n"
