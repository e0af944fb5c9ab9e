"""Extract the reference's golden values used to pin the oracle.

Reads UppASD's own regression definitions (tests/regulartests.yaml in the
reference tree) as text -- PyYAML is not needed -- and writes
``reference_pins.json`` next to this script.  Run it where the reference tree
is available:

    python tests/golden/make_golden.py /path/to/UppASD/tests/regulartests.yaml

Only the uncommented ``expected:`` line of each selected block is kept; the
commented-out history in the YAML is ignored.
"""
import json
import os
import re
import sys

CASES = [
    # (name, workingdir, outfile, select value, comparison)
    ("solvers_midpoint", "./Solvers", "averages.1", 8000, "similar"),
    ("solvers_heun", "./Solvers", "averages.4", 8000, "similar"),
    ("solvers_depondt", "./Solvers", "averages.5", 8000, "similar"),
    ("bccfe_sd_iter0", "./bccFe/", "./averages.S", 0, "similar"),
    ("bccfe_sd_iter2700", "./bccFe/", "./averages.S", 2700, "similar"),
    ("bccfe_sd_cumulants", "./bccFe/", "./cumulants.S", 41, "similar"),
    ("bccfe_mc_iter0", "./bccFe/", "./averages.M", 0, "similar"),
    ("bccfe_mc_iter2700", "./bccFe/", "./averages.M", 2700, "similar"),
    ("bccfe_mc_cumulants", "./bccFe/", "./cumulants.M", 41, "similar"),
    ("bccfe_hb_iter0", "./bccFe/", "./averages.H", 0, "sloppy"),
    ("bccfe_hb_iter2700", "./bccFe/", "./averages.H", 2700, "sloppy"),
]


def extract(text, workingdir, outfile, select):
    lines = text.splitlines()
    out = None
    in_case = False
    in_file = False
    for n, ln in enumerate(lines):
        s = ln.strip()
        if s.startswith("- workingdir:"):
            in_case = workingdir in s
            in_file = False
        elif in_case and s.startswith("- outfile:"):
            in_file = s.split(":", 1)[1].strip() == outfile
        elif in_case and in_file and re.match(r'"#_Iter\.":\s*%d\s*$' % select, s):
            extract_line = None
            for m in range(n + 1, min(n + 30, len(lines))):
                t = lines[m].strip()
                if t.startswith("extract:") and extract_line is None:
                    extract_line = json.loads(t.split(":", 1)[1].strip())
                if t.startswith("expected:"):
                    vals = json.loads(t.split(":", 1)[1].strip())
                    out = {"extract": extract_line, "expected": vals}
                    break
            break
    if out is None:
        raise SystemExit(f"not found: {workingdir} {outfile} {select}")
    return out


def read_inputs(testdir):
    """Scenario inputs from the reference's test directories (jfile, momfile, inpsd)."""
    def rows(fn):
        out = []
        for ln in open(os.path.join(testdir, fn)):
            t = ln.split()
            if t and not t[0].startswith("#"):
                out.append(t)
        return out

    def keys(fn):
        d = {}
        for t in rows(fn):
            d.setdefault(t[0].lower(), t[1:])
        return d

    sol = keys("Solvers/inpsd.dat.base")
    sj = rows("Solvers/jfile")[0]
    sm = rows("Solvers/momfile")[0]
    bfe = keys("bccFe/inpsd.dat.base")
    bj = rows("bccFe/jfile")
    bm = rows("bccFe/momfile")[0]
    return {
        "solvers": {"ncell": [int(v) for v in sol["ncell"][:3]], "j_mry": float(sj[5]),
                    "mom": float(sm[2]), "damping": float(sol["damping"][0]),
                    "timestep": float(sol["timestep"][0]), "temp": float(sol["temp"][0]),
                    "tseed_default": 1, "nstep_checked": 8000,
                    "source": "tests/Solvers/{inpsd.dat.base,jfile,momfile}"},
        "bccfe": {"ncell": [int(v) for v in bfe["ncell"][:3]],
                  "shell_vectors": [[float(v) for v in r[2:5]] for r in bj],
                  "j_mry": [float(r[5]) for r in bj], "mom": float(bm[2]),
                  "emom0": [float(v) for v in bm[3:6]], "tseed": int(bfe["tseed"][0]),
                  "ip_nstep": 2000, "ip_temp": 500.0, "ip_timestep": 1.0e-16, "ip_damping": 0.5,
                  "temp": float(bfe["temp"][0]), "damping": float(bfe["damping"][0]),
                  "timestep_default_real4": 1.0e-16, "avrg_step": int(bfe["avrg_step"][0]),
                  "cumu_step": int(bfe["cumu_step"][0]), "cumu_buff": int(bfe["cumu_buff"][0]),
                  "source": "tests/bccFe/{inpsd.dat.base,jfile,momfile}; Input/inputdata.f90:457"},
    }


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else "regulartests.yaml"
    text = open(src).read()
    pins = {"inputs": read_inputs(os.path.dirname(os.path.abspath(src)))}
    for name, wd, of, sel, cmp in CASES:
        e = extract(text, wd, of, sel)
        e["comparison"] = cmp
        e["source"] = f"tests/regulartests.yaml {wd} {of} #_Iter.={sel}"
        pins[name] = e
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_pins.json")
    with open(dst, "w") as f:
        json.dump(pins, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    main()
