"""Generate conductor_ior.py: the RGB eta and k of the conductor names the
reference's scene files may use (material="gold" ...), from the reference's
own spectral data and CIE tables, converted the way the reference converts
them.

IORHelper::evalConductorIOR (tools/Common.cpp:44-81) maps the names to
data/IOR/<name>.{eta,k}.spd and reads each file with
extractAndConvertSpectrumFromFile (lines 83-110): (wavelength, value) pairs,
'#' lines skipped.  Color3::setFromSampledSpectrum (core/Color.cpp:423-442)
then integrates the spectrum against the CIE 1931 matching functions at the
471 wavelengths of the reference's tables (linear interpolation of the
samples, pbrt's InterpolateSpectrumSamples), scales by
(lambda_last - lambda_first) / (CIE_Y_INTEGRAL * 471) and converts XYZ to
linear RGB with the reference's matrix, clamping negatives to zero
(Color.h:196-205).  This script restates those steps in binary32 and reads
the tables and the data from the reference tree; it writes only the
resulting 48 numbers.

    python raytracer_gb300/make_conductor_ior.py /path/to/RaytracerNew2
"""
import os
import re
import sys

import numpy as np

F = np.float32
NAMES = {"gold": "Au", "silver": "Ag", "aluminium": "Al", "copper": "Cu", "chromium": "Cr", "iron": "Fe",
         "nickel": "Ni_palik", "tin": "SnTe_palik"}   # tools/Common.cpp:44-54


def _table(src, name):
    m = re.search(r"const\s+real\s+colorSpace::%s\s*\[[^\]]*\]\s*=\s*\{(.*?)\};" % name, src, re.S)
    if not m:
        raise SystemExit("table %s not found" % name)
    body = re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S))
    vals = [F(v.strip().rstrip("fF")) for v in body.replace("\n", " ").split(",") if v.strip()]
    return np.array(vals, F)


_NUM = re.compile(r"[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?")


def _num(tok):
    """tools::stringToNum<float>: istringstream >> float, which reads the
    longest numeric prefix and leaves 0 when there is none (C++11)."""
    m = _NUM.match(tok)
    return F(m.group(0)) if m else F(0)


def _read_spd(path):
    """extractAndConvertSpectrumFromFile's reading: every line that does not
    start with '#' gives a (wavelength, value) pair, header lines and empty
    lines included (as zeros)."""
    lam, val = [], []
    for line in open(path, encoding="latin-1").read().split("\n"):
        if line.endswith("\r"):
            line = line[:-1]
        if line[:1] == "#":
            continue
        toks = line.split() + ["", ""]
        lam.append(_num(toks[0]))
        val.append(_num(toks[1]))
    if open(path, "rb").read().endswith(b"\n"):   # getline gives no line after a final newline
        lam.pop()
        val.pop()
    return np.array(lam, F), np.array(val, F)


def _interp(lam, val, l):
    """pbrt's InterpolateSpectrumSamples in binary32."""
    n = len(lam)
    if l <= lam[0]:
        return val[0]
    if l >= lam[n - 1]:
        return val[n - 1]
    first, length = 0, n
    while length > 0:
        half = length >> 1
        mid = first + half
        if lam[mid] <= l:
            first = mid + 1
            length -= half + 1
        else:
            length = half
    off = min(max(first - 1, 0), n - 2)
    t = F((l - lam[off]) / (lam[off + 1] - lam[off]))
    return F(F(F(1) - t) * val[off]) + F(t * val[off + 1])


def spectrum_to_rgb(lam, val, cie):
    cl, cx, cy, cz = cie
    xyz = [F(0), F(0), F(0)]
    for i in range(len(cl)):
        v = _interp(lam, val, cl[i])
        xyz[0] = F(xyz[0] + F(v * cx[i]))
        xyz[1] = F(xyz[1] + F(v * cy[i]))
        xyz[2] = F(xyz[2] + F(v * cz[i]))
    scale = F(F(cl[-1] - cl[0]) / F(F(106.856895) * F(len(cl))))
    x, y, z = (F(c * scale) for c in xyz)
    r = F(F(F(3.240479) * x) - F(F(1.537150) * y)) - F(F(0.498535) * z)
    g = F(F(F(-0.969256) * x) + F(F(1.875991) * y)) + F(F(0.041556) * z)
    b = F(F(F(0.055648) * x) - F(F(0.204043) * y)) + F(F(1.057311) * z)
    return tuple(float(max(F(0), F(c))) for c in (r, g, b))


def compute(ref_root):
    """{name: (eta rgb, k rgb)} from the reference tree."""
    src = open(os.path.join(ref_root, "src", "core", "Color.cpp"), encoding="latin-1").read()
    cie = (_table(src, "CIE_lambda"), _table(src, "CIE_X"), _table(src, "CIE_Y"), _table(src, "CIE_Z"))
    assert all(len(t) == 471 for t in cie)
    out = {}
    for name, tech in NAMES.items():
        base = os.path.join(ref_root, "data", "IOR", tech)
        out[name] = (spectrum_to_rgb(*_read_spd(base + ".eta.spd"), cie),
                     spectrum_to_rgb(*_read_spd(base + ".k.spd"), cie))
    return out


def main(ref_root):
    rows = []
    for name, (eta, k) in compute(ref_root).items():
        rows.append('    "%s": ((%r, %r, %r), (%r, %r, %r)),' % ((name,) + eta + k))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "conductor_ior.py")
    with open(out, "w") as f:
        f.write('"""RGB (eta, k) of the conductor names of reference scene files (material="gold" ...).\n\n'
                "Generated by make_conductor_ior.py from the reference's data/IOR spectra with\n"
                "its conversion (Color3::setFromSampledSpectrum, core/Color.cpp:423-442).\n"
                '"""\n\nMATERIALS = {\n' + "\n".join(rows) + "\n}\n")
    print(out)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("RT_REFERENCE_ROOT")
    if not root or not os.path.isdir(os.path.join(root, "data", "IOR")):
        raise SystemExit("usage: make_conductor_ior.py <reference>/RaytracerNew2 "
                         "(or set RT_REFERENCE_ROOT): the directory holding src/ and data/IOR/")
    main(root)
