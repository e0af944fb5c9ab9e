"""Extract the reference's golden values used to pin the oracle.

Reads UppASD's own regression definitions (tests/regulartests.yaml and
tests/cudatests.yaml in the reference tree) as text -- PyYAML is not needed -- and writes
``reference_pins.json`` next to this script.  Run it where the reference tree
is available:

    python tests/golden/make_golden.py /path/to/UppASD/tests/regulartests.yaml

Only the uncommented ``expected:`` line of each selected block is kept; the
commented-out history in the YAML is ignored.
"""
import json
import os
import re
import struct
import sys

CASES = [
    # (name, workingdir, outfile, select value (iteration, or iteration and projection), comparison)
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
    ("heisstripe_iter1190", "./HeisStripe", "averages.HeisStri.out", 1190, "similar"),
    ("heisstripe_energy1460", "./HeisStripe", "./totenergy.HeisStri.out", 1460, "similar"),
    ("kagome_iter13000", "./kagome", "averages.kagome_T.out", 13000, "similar"),
    ("kagome_traj2400", "./kagome", "trajectory.kagome_T.001.1.out", 2400, "similar"),
    ("heischain_iter1000", "./HeisChain", "averages.HeisWire.out", 1000, "similar"),
    ("heischain_energy1400", "./HeisChain", "totenergy.HeisWire.out", 1400, "similar"),
    ("heischainaf_iter1000", "./HeisChainAF", "./averages.AF_WireT.out", 1000, "similar"),
    ("heischainaf_proj5000_type1", "./HeisChainAF", "./projavgs.AF_WireT.out", (5000, 1), "similar"),
    ("heischainaf_proj5000_type2", "./HeisChainAF", "./projavgs.AF_WireT.out", (5000, 2), "similar"),
    ("heischainaf_energy1500", "./HeisChainAF", "./totenergy.AF_WireT.out", 1500, "similar"),
    ("feco_iter4700", "./FeCo/", "./averages.test", 4700, "sloppy"),
    ("feco_cumulants221", "./FeCo/", "./cumulants.test", 221, "sloppy"),
    ("scsurf_iter800", "./SCsurf", "averages.SCsurf_T.out", 800, "similar"),
    ("kagome_cuda_iter1300", "./kagome_cuda", "averages.kagome_T.out", 1300, "similar"),
    ("kagome_cuda_cumulants171", "./kagome_cuda", "cumulants.kagome_T.out", 171, "similar"),
    ("feco_cuda_iter4700", "./FeCo_cuda/", "./averages.test", 4700, "sloppy"),
    ("feco_cuda_cumulants221", "./FeCo_cuda/", "./cumulants.test", 221, "sloppy"),
    ("bccfe_cuda_iter1700", "./bccFe_cuda/", "./averages.test", 1700, "sloppy"),
    ("bccfe_cuda_cumulants41", "./bccFe_cuda/", "./cumulants.test", 41, "sloppy"),
]


def _bracketed(line):
    """The [...] list of a YAML `key: [...]  # comment` line."""
    v = line.split(":", 1)[1]
    return v[v.index("["):v.rindex("]") + 1]


def extract(text, workingdir, outfile, select):
    select, atom = select if isinstance(select, tuple) else (select, None)
    lines = text.splitlines()
    out = None
    in_case = False
    in_file = False
    for n, ln in enumerate(lines):
        s = ln.strip()
        if s.startswith("- workingdir:"):
            in_case = s.split(":", 1)[1].split("#")[0].strip().strip('"') == workingdir
            in_file = False
        elif in_case and s.startswith("- outfile:"):
            in_file = s.split(":", 1)[1].strip() == outfile
        elif in_case and in_file and re.match(r'"#_Iter\."\s*:\s*%d\s*(#.*)?$' % select, s):
            if atom is not None and not re.match(r'"#_Atom"\s*:\s*%d\s*(#.*)?$' % atom, lines[n + 1].strip()):
                continue
            extract_line = None
            for m in range(n + 1, min(n + 30, len(lines))):
                t = lines[m].strip()
                if t.startswith("extract:") and extract_line is None:
                    extract_line = json.loads(_bracketed(t))
                if t.startswith("expected:"):
                    vals = json.loads(_bracketed(t))
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

    def nums(fn):
        return [[float(v.replace("d", "e").replace("D", "e")) for v in r] for r in rows(fn)]

    def system(d):
        """Keywords and the tables they name in one test directory."""
        k = keys(d + "/inpsd.dat")
        lines = [ln.split() for ln in open(os.path.join(testdir, d, "inpsd.dat"))]
        heads = [t[0].lower() if t else "" for t in lines]
        c0 = heads.index("cell")
        cell = [[float(v) for v in lines[c0][1:4]]] + [[float(v) for v in lines[c0 + q][0:3]] for q in (1, 2)]
        pos = {int(r[0]): r for r in nums(d + "/" + os.path.basename(k["posfile"][0]))}
        mom = {int(r[0]): r for r in nums(d + "/" + os.path.basename(k["momfile"][0]))}
        sites = [[pos[i][1]] + pos[i][2:5] + mom[i][2:6] for i in sorted(pos)]
        out = {"ncell": [int(v) for v in k["ncell"][:3]], "bc": k["bc"][:3], "cell": cell,
               "sym": int(k.get("sym", ["0"])[0]), "sites": sites,
               "jfile": nums(d + "/" + os.path.basename(k["exchange"][0])),
               "damping": float(k["damping"][0]), "temp": float(k["temp"][0]),
               # without the keyword, delta_t keeps its default, a REAL(4) literal (Input/inputdata.f90:457)
               "timestep": (float(k["timestep"][0].replace("d", "e")) if "timestep" in k
                            else struct.unpack("f", struct.pack("f", 1.0e-16))[0]),
               "nstep": int(k["nstep"][0]),
               "initmag": int(k["initmag"][0]), "sdealgh": int(k.get("sdealgh", ["1"])[0]),
               "do_reduced": k.get("do_reduced", ["N"])[0].upper() == "Y", "tseed_default": 1,
               "maptype": int(k.get("maptype", ["1"])[0]),
               "aunits": k.get("aunits", ["N"])[0].upper() == "Y",
               "posfiletype": k.get("posfiletype", ["C"])[0].upper(),
               "do_jtensor": int(k.get("do_jtensor", ["0"])[0]),
               "source": f"tests/{d}/inpsd.dat and the files it names"}
        if "dm" in k:
            out["dmfile"] = nums(d + "/" + os.path.basename(k["dm"][0]))
        if "anisotropy" in k:
            out["kfile"] = nums(d + "/" + os.path.basename(k["anisotropy"][0]))
        if "ip_nphase" in heads and k.get("ip_mode", ["N"])[0].upper() == "S":
            q = heads.index("ip_nphase")
            out["ip_phases"] = [[float(v.replace("d", "e")) for v in lines[q + 1 + p][:4]]
                                for p in range(int(lines[q][1]))]
        if "restartfile" in k:
            rs = nums(d + "/" + os.path.basename(k["restartfile"][0]))
            out["restart"] = [r[3:7] for r in rs]   # |m|, m_x, m_y, m_z per atom
        return out

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
        "heisstripe": system("HeisStripe"),
        "kagome": system("kagome"),
        "heischain": system("HeisChain"),
        "heischainaf": system("HeisChainAF"),
        "scsurf": system("SCsurf"),
        "feco_cuda": dict(system("FeCo_cuda"), cumu_step=int(keys("FeCo_cuda/inpsd.dat")["cumu_step"][0]),
                          cumu_buff=int(keys("FeCo_cuda/inpsd.dat")["cumu_buff"][0]),
                          avrg_step=int(keys("FeCo_cuda/inpsd.dat").get("avrg_step", ["100"])[0])),
        "bccfe_cuda": dict(system("bccFe_cuda"), cumu_step=int(keys("bccFe_cuda/inpsd.dat")["cumu_step"][0]),
                           cumu_buff=int(keys("bccFe_cuda/inpsd.dat")["cumu_buff"][0]),
                           avrg_step=int(keys("bccFe_cuda/inpsd.dat")["avrg_step"][0])),
        "kagome_cuda": dict(system("kagome_cuda"), cumu_step=int(keys("kagome_cuda/inpsd.dat")["cumu_step"][0]),
                            cumu_buff=int(keys("kagome_cuda/inpsd.dat")["cumu_buff"][0]),
                            avrg_step=int(keys("kagome_cuda/inpsd.dat")["avrg_step"][0])),
        "feco": dict(system("FeCo"), cumu_step=int(keys("FeCo/inpsd.dat")["cumu_step"][0]),
                     cumu_buff=int(keys("FeCo/inpsd.dat")["cumu_buff"][0]),
                     avrg_step=int(keys("FeCo/inpsd.dat").get("avrg_step", ["100"])[0])),
    }


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else "regulartests.yaml"
    # the GPU cases of the suite live in a second file beside it
    text = open(src).read() + "\n" + open(os.path.join(os.path.dirname(os.path.abspath(src)), "cudatests.yaml")).read()
    pins = {"inputs": read_inputs(os.path.dirname(os.path.abspath(src)))}
    for name, wd, of, sel, cmp in CASES:
        e = extract(text, wd, of, sel)
        e["comparison"] = cmp
        yaml = "cudatests.yaml" if "_cuda" in wd else "regulartests.yaml"
        e["source"] = f"tests/{yaml} {wd} {of} #_Iter.={sel}" if not isinstance(sel, tuple) else \
            f"tests/{yaml} {wd} {of} #_Iter.={sel[0]} #_Atom={sel[1]}"
        pins[name] = e
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_pins.json")
    with open(dst, "w") as f:
        json.dump(pins, f, indent=1)
    print("wrote", dst)


if __name__ == "__main__":
    main()
