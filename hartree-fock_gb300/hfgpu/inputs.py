"""Reader of the reference program's input format ($molecule / $scf / $basis; src/Input.cpp:23-416).

Blocks may come in any order; tokens are case-insensitive; '#' starts a comment.  $molecule: charge,
multiplicity, then `symbol-or-Z x y z` (bohr).  $basis: one basis name.  $scf: `KEYWORD value` pairs
with the reference's keyword set and defaults (SCF.hpp:9-32, Input.cpp:127-140).
"""
from __future__ import annotations

from dataclasses import dataclass, field

SYMBOL_Z = {"h": 1, "he": 2, "li": 3, "be": 4, "b": 5, "c": 6, "n": 7, "o": 8, "f": 9, "ne": 10}

_FLOAT = {"energy_tol", "density_tol", "diis_tol", "schwartz_thresh", "density_thresh", "symmetry_tol",
          "stop_damp_thresh", "level_shift", "lshift_gap_tol", "stop_lshift_thresh"}
_INT = {"max_iter", "diis_size", "damp", "max_damp_cycles", "max_lshift_cycles"}
_BOOL = {"diis", "direct", "symmetry", "print_full_mos", "unrestricted"}


@dataclass
class JobInput:
    charge: int
    multiplicity: int
    Z: list
    xyz: list
    basis: str
    scf: dict = field(default_factory=dict)  # lower-case keyword -> value, as set in the file


def _bool(tok: str, key: str) -> bool:
    t = tok.lower()
    if t in ("true", "1"):
        return True
    if t in ("false", "0"):
        return False
    raise ValueError(f"Invalid boolean value for {key} in $scf block: {tok}")


def parse(text: str) -> JobInput:
    blocks = {"molecule": [], "scf": [], "basis": []}
    cur = None
    for lineno, line in enumerate(text.splitlines(), 1):
        for tok in line.split():
            if tok.startswith("#"):
                break
            lt = tok.lower()
            if lt in ("$molecule", "$scf", "$basis"):
                cur = lt[1:]
            elif lt == "$end":
                cur = None
            elif cur is None:
                raise ValueError(f"Unexpected token at line {lineno}: {tok}")
            else:
                blocks[cur].append(tok)
    mol = blocks["molecule"]
    if len(mol) < 2:
        raise ValueError("Invalid charge in $molecule block.")
    charge, mult = int(mol[0]), int(mol[1])
    Z, xyz = [], []
    rest = mol[2:]
    if len(rest) % 4 != 0:
        raise ValueError("Incomplete atom specification in $molecule block.")
    for k in range(0, len(rest), 4):
        a = rest[k]
        Z.append(int(a) if a.isdigit() else SYMBOL_Z[a.lower()])
        xyz.append([float(v) for v in rest[k + 1:k + 4]])
    if not Z:
        raise ValueError("No atoms specified in $molecule block.")
    if len(blocks["basis"]) != 1:
        raise ValueError("Error in basis set specification in $basis block.")
    scf = {}
    toks = blocks["scf"]
    if len(toks) % 2:
        raise ValueError("Error reading value for option: " + toks[-1])
    for k in range(0, len(toks), 2):
        key, val = toks[k].lower(), toks[k + 1]
        if key in _FLOAT:
            scf[key] = float(val)
        elif key in _INT:
            scf[key] = int(val)
        elif key in _BOOL:
            scf[key] = _bool(val, toks[k])
        elif key == "guess_mix":
            scf[key] = 1 if val.lower() == "true" else (0 if val.lower() == "false" else int(val))
        else:
            raise ValueError("Unknown option in $scf block: " + toks[k])
    return JobInput(charge, mult, Z, xyz, blocks["basis"][0], scf)


def check_supported(job: JobInput, input_frame: bool = False) -> None:
    """Rejects the keywords whose reference semantics this engine does not reproduce, instead of ignoring
    them: SYMMETRY TRUE (the default; the reference translates to the centre of mass and rotates into the
    point-group frame, src/Molecule.cpp:19-27) unless the caller accepts the input frame."""
    if job.scf.get("symmetry", True) and not input_frame:
        raise ValueError("SYMMETRY TRUE (the reference's default) reorients the molecule into its point-group "
                         "frame (src/Molecule.cpp:19-27), which this engine does not do: set SYMMETRY FALSE in "
                         "$scf, or run with input_frame=True to compute in the input frame (same energy; "
                         "densities and gradients in the input frame)")


def scf_options(job: JobInput, precision: int = 0, fp32_cutoff: float = 2e-4, full_rebuild_every: int = 0) -> dict:
    """The hfg_scf_options fields for a parsed job, with the reference's defaults."""
    s = job.scf
    max_iter = s.get("max_iter", 30)
    return dict(
        max_iter=max_iter, energy_tol=s.get("energy_tol", 1e-6), density_tol=s.get("density_tol", 1e-6),
        use_diis=int(s.get("diis", True)), diis_size=s.get("diis_size", 6), diis_tol=s.get("diis_tol", 1e-6),
        unrestricted=int(s.get("unrestricted", job.multiplicity != 1)), guess_mix=s.get("guess_mix", 0),
        damp=s.get("damp", 0), max_damp_iter=s.get("max_damp_cycles", max_iter),
        stop_damp_thresh=s.get("stop_damp_thresh", 0.0), level_shift=s.get("level_shift", 0.0),
        lshift_gap_tol=s.get("lshift_gap_tol", float("inf")), max_lshift_iter=float(s.get("max_lshift_cycles", max_iter)),
        stop_lshift_thresh=s.get("stop_lshift_thresh", 0.0), schwartz_threshold=s.get("schwartz_thresh", 1e-10),
        density_threshold=s.get("density_thresh", 1e-10), precision=precision, fp32_cutoff=fp32_cutoff,
        full_rebuild_every=full_rebuild_every, verbose=0, direct=int(s.get("direct", True)))
