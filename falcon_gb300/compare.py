"""Per-variable error of one state against another (mixed precision against
the FP64 path), as the reference's own checks would state it: over the
interior cells of every block, for each evolved variable,

    rel_l2  = ||u - ref||_2 / ||ref||_2     (the RMS error over the RMS value)
    rel_max = max|u - ref| / max|ref|       (norm-wise maximum error)

States are host arrays in the falcon_download_state layout
[block][FALCON_NVAR][k][j][i] with ng ghost layers. Variables whose reference
is identically zero report 0 for both (and `active` False).
"""
import numpy as np

from .config import NVAR_EVOLVED, VAR_NAMES


def state_errors(u, ref, ng=2, nvar=NVAR_EVOLVED):
    """{var name: {"rel_l2", "rel_max", "active"}} over the interior cells."""
    out = {}
    sl = (slice(None), slice(ng, -ng), slice(ng, -ng), slice(ng, -ng))
    for v in range(nvar):
        a = u[:, v][sl]
        b = ref[:, v][sl]
        d = a - b
        nb = float(np.sqrt(np.square(b).sum()))
        mb = float(np.abs(b).max())
        active = mb > 0.0
        out[VAR_NAMES[v]] = {
            "rel_l2": float(np.sqrt(np.square(d).sum())) / nb if active else 0.0,
            "rel_max": float(np.abs(d).max()) / mb if active else 0.0,
            "active": bool(active),
        }
    return out


def worst(errors, key):
    """The largest `key` over the active variables."""
    vals = [e[key] for e in errors.values() if e["active"]]
    return max(vals) if vals else 0.0
