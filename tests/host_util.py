"""Helpers for the C++ host mirror tests: build the test driver, write CFG files."""
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "latticemontecarlo_gb300"
EXE = PKG / "bin" / "lmc_gb300"
CHECK = PKG / "bin" / "host_check"
MASS = {"X": 0.0, "Al": 26.98, "Mg": 24.31, "Zn": 65.38, "Cu": 63.55, "Sn": 118.71}


def build_check() -> Path:
    src = [ROOT / "tests" / "host" / "host_check.cpp", PKG / "host" / "lmc_host.cpp"]
    inputs = src + [PKG / "host" / "lmc_host.hpp", PKG / "liblmc_gb300.so"]
    if not CHECK.exists() or CHECK.stat().st_mtime < max(p.stat().st_mtime for p in inputs):
        zlib = subprocess.run(["g++", "-x", "c++", "-E", "-"], input="#include <zlib.h>\n", capture_output=True,
                              text=True).returncode == 0
        subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(PKG / "host"), *map(str, src), "-o", str(CHECK),
                        "-L", str(PKG), "-llmc_gb300", "-Wl,-rpath,$ORIGIN/..", *(["-lz"] if zlib else [])],
                       check=True)
    return CHECK


def write_cfg(path, n: int, species: np.ndarray, alphabet) -> None:
    """CFG text with atom i on lattice id i (relative positions from the closed-form ids)."""
    ids = np.arange(4 * n ** 3)
    plane = 2 * n * n
    hx = ids // plane
    rem = ids - hx * plane
    hy = rem // n
    hz = 2 * (rem - hy * n) + ((hx + hy) & 1)
    L = n * 4.046
    lines = [f"Number of particles = {ids.size}", "A = 1.0 Angstrom (basic length-scale)"]
    for i in range(3):
        for j in range(3):
            lines.append(f"H0({i + 1},{j + 1}) = {L if i == j else 0} A")
    lines += [".NO_VELOCITY.", "entry_count = 6", "auxiliary[0] = ix", "auxiliary[1] = iy", "auxiliary[2] = iz"]
    for k in range(ids.size):
        el = alphabet[int(species[k])]
        lines.append(f"{MASS[el]}\n{el}\n{hx[k] / (2 * n)} {hy[k] / (2 * n)} {hz[k] / (2 * n)} 0 0 0")
    Path(path).write_text("\n".join(lines) + "\n")
