"""input.file parser with the reference's semantics (MC/tools/fileTools.py:8-46).

`key : value  # comment` lines.  String keys: mode, material, elastic,
Bethe_model.  Integer keys: num_el, maxScatt.  Keys containing 'output' are
comma lists.  gen_tables and diffMFP are booleans (true when the value
contains 'es', as in 'yes').  Every other key is a float.  Lines starting with
'#' and empty lines are skipped; a value keeps everything before an inline '#'.
"""

STRING_KEYS = ("mode", "material", "elastic", "Bethe_model")
INT_KEYS = ("num_el", "maxScatt")
BOOL_KEYS = ("gen_tables", "diffMFP")


def parse_input(text):
    data = {}
    for line in text.split("\n"):
        if not line.strip() or line.startswith("#"):
            continue
        line = line.partition("#")[0]
        parts = [p.strip(" ") for p in line.split(":")]
        key = parts[0]
        if key in STRING_KEYS:
            data[key] = parts[1]
        elif key in INT_KEYS:
            data[key] = int(parts[1])
        elif "output" in key:
            data[key] = parts[1].replace(" ", "").split(",")
        elif key in BOOL_KEYS:
            data[key] = "es" in parts[1]
        else:
            data[key] = float(parts[1])
    return data


def readInput(fileName="input.file"):  # noqa: N802 - the reference's name
    """Read parameters from an input file (MC/tools/fileTools.py:8)."""
    with open(fileName) as f:
        return parse_input(f.read())


# Defaults for keys the trajectory needs but older input files omit (the
# reference raises KeyError for them: MC/tools/multiScatter.py:110).
# maxScatt bounds every trajectory (and so every kernel): a continuous-mode
# electron below J/1.166 gains energy under the Bethe law and would otherwise
# only end by leaving the sample.
DEFAULTS = {
    "thickness": 1e30,
    "diffMFP": False,
    "maxScatt": 10 ** 6,
    "elastic": "Ruth_vanilla",
    "Bethe_model": "classical",
    "mode": "DS",
    "s_tilt": 0.0,
    "Wc": 100.0,
    "tol_E": 1e-3,
    "tol_W": 1e-3,
}


def with_defaults(input_par):
    out = dict(DEFAULTS)
    out.update(input_par)
    return out
