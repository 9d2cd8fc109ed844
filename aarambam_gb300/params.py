"""Parameter-file reader for the 2LPT initial-condition generator.

Mirrors read_parameterfile (Aarambam/LPT/Basis/read_param.c:8-262): a fixed
tag table, every tag required exactly once, lines whose first token starts
with '%' ignored, the second whitespace-separated token converted with C
atof / atoi semantics (leading numeric prefix, 0 when there is none), unknown
or repeated tags and missing tags reported with the reference's messages.
The reference prints those messages and exits with status 0
(read_param.c:251-255); here they are collected on a ParameterError and the
command-line entry point reproduces the print-and-exit behaviour.
"""
from __future__ import annotations

import re

FLOAT, STRING, INT = 1, 2, 3

# tag -> type, in the reference's declaration order (read_param.c:25-184)
TAGS = [
    ("Omega", FLOAT), ("OmegaLambda", FLOAT), ("OmegaBaryon", FLOAT), ("OmegaDM_2ndSpecies", FLOAT),
    ("HubbleParam", FLOAT), ("ShapeGamma", FLOAT), ("Sigma8", FLOAT), ("PrimordialIndex", FLOAT),
    ("Box", FLOAT), ("Redshift", FLOAT), ("Fnl", FLOAT), ("N_modes", INT), ("FileWithAlphaCoeff", STRING),
    ("FileWithX0Coeff", STRING), ("SavePotentialField", INT), ("FixedAmplitude", INT), ("PhaseFlip", INT),
    ("Nmesh", INT), ("Nsample", INT), ("Nmax", INT), ("GlassFile", STRING), ("FileWithInputSpectrum", STRING),
    ("FileWithInputTransfer", STRING), ("GlassTileFac", INT), ("Seed", INT), ("SphereMode", INT),
    ("NumFilesWrittenInParallel", INT), ("OutputDir", STRING), ("FileBase", STRING), ("WhichSpectrum", INT),
    ("WhichTransfer", INT), ("UnitVelocity_in_cm_per_s", FLOAT), ("UnitLength_in_cm", FLOAT),
    ("UnitMass_in_g", FLOAT), ("InputSpectrum_UnitLength_in_cm", FLOAT), ("WDM_On", INT),
    ("WDM_Vtherm_On", INT), ("WDM_PartMass_in_kev", FLOAT),
]
TAG_TYPES = dict(TAGS)

# 2LPTResBasis adds the P(k) oscillation after SavePotentialField
# (Aarambam/LPT/ResBasis/read_param.c:88-99)
_at = [t for t, _ in TAGS].index("SavePotentialField") + 1
TAGS_RESBASIS = TAGS[:_at] + [("A_res", FLOAT), ("w_res", FLOAT), ("phi_res", FLOAT)] + TAGS[_at:]
TAG_TABLES = {"basis": TAGS, "resbasis": TAGS_RESBASIS}

_FLOAT_PREFIX = re.compile(r"^\s*[+-]?((\d+\.?\d*)|(\.\d+))([eE][+-]?\d+)?")
_INT_PREFIX = re.compile(r"^\s*[+-]?\d+")


class ParameterError(Exception):
    """Raised with the list of messages the reference would have printed."""

    def __init__(self, messages):
        super().__init__("\n".join(messages))
        self.messages = list(messages)


def c_atof(s: str) -> float:
    """C atof: longest valid leading number, 0.0 when none (also inf/nan words)."""
    t = s.strip().lower()
    for word, val in (("infinity", float("inf")), ("inf", float("inf")), ("nan", float("nan"))):
        for sign, mul in (("", 1), ("+", 1), ("-", -1)):
            if t.startswith(sign + word):
                return mul * val
    m = _FLOAT_PREFIX.match(s)
    return float(m.group(0)) if m else 0.0


def c_atoi(s: str) -> int:
    """C atoi: leading decimal integer, 0 when none (wraps like a 32-bit int)."""
    m = _INT_PREFIX.match(s)
    if not m:
        return 0
    v = int(m.group(0))
    return (v + 2**31) % 2**32 - 2**31


def parse_parameter_text(text: str, fname: str = "<text>", variant: str = "basis") -> dict:
    """Parse parameter-file text with the tag table of `variant` ("basis" or
    "resbasis").  Returns {tag: value}; raises ParameterError."""
    tags = TAG_TABLES[variant]
    types = dict(tags)
    remaining = {t for t, _ in tags}
    values: dict = {}
    errors = []
    # fgets(buf, 200, fd): a physical line longer than 199 characters is read in
    # 199-character pieces, each parsed on its own
    pieces = []
    for line in text.splitlines(keepends=True):
        while len(line) > 199:
            pieces.append(line[:199])
            line = line[199:]
        pieces.append(line)
    for piece in pieces:
        toks = piece.split()
        if len(toks) < 2:
            continue
        tag, val = toks[0], toks[1]
        if tag.startswith("%"):
            continue
        if tag in remaining:
            remaining.discard(tag)
            kind = types[tag]
            values[tag] = c_atof(val) if kind == FLOAT else c_atoi(val) if kind == INT else val
        else:
            errors.append(f"Error in file {fname}:   Tag '{tag}' not allowed or multiple defined.")
    for tag, _ in tags:
        if tag in remaining:
            errors.append(f"Error. I miss a value for tag '{tag}' in parameter file '{fname}'.")
    if errors:
        raise ParameterError(errors)
    return values


def read_parameterfile(fname: str, variant: str = "basis") -> dict:
    """Read a 2LPT parameter file (read_param.c:8-262)."""
    try:
        with open(fname, "r", errors="surrogateescape") as f:
            text = f.read()
    except OSError:
        raise ParameterError([f"Parameter file {fname} not found."]) from None
    return parse_parameter_text(text, fname, variant)
