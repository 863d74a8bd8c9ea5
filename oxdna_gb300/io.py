"""oxDNA file formats and input keys, host side.

* topology files, both layouts the reference reads
  (src/Utilities/TopologyParser.cpp:52-130 old "strand base n3 n5" lines, and the new
  "N n_strands 5->3" layout of src/Interactions/DNAInteraction.cpp:1508-1560);
* configuration files (src/Backends/SimBackend.cpp:600-650: "t = ", "b = ", "E = " header,
  then one "pos a1 a3 [v L]" line per nucleotide), read and written in double precision;
* `key = value` input files (src/Utilities/parse_input/) and the temperature syntax of
  Utils::get_temperature (src/Utilities/Utils.cpp:316-352).

Only numpy is needed; nothing here touches the GPU.
"""

from __future__ import annotations

import dataclasses
import math
import re
from typing import Dict, List, Optional

import numpy as np

# base codes: N_A = 0, N_G = 1, N_C = 2, N_T = 3, N_DUMMY = 4 (src/defs.h)
BASE_CODE = {"A": 0, "G": 1, "C": 2, "T": 3, "U": 3, "D": 4}
BASE_CHAR = {0: "A", 1: "G", 2: "C", 3: "T", 4: "D"}


class OxDNAFormatError(ValueError):
    """Raised for malformed topology, configuration or input files."""


def type_from_btype(btype: int) -> int:
    """Base type (0..3) of a pairing code, as the reference maps integer codes."""
    return btype % 4 if btype >= 0 else 3 - ((3 - btype) % 4)


@dataclasses.dataclass
class Topology:
    n3: np.ndarray  # int32 [N], index of the 3' neighbour or -1
    n5: np.ndarray  # int32 [N], index of the 5' neighbour or -1
    btype: np.ndarray  # int32 [N], pairing code (A+T = G+C = 3)
    type: np.ndarray  # int32 [N], base type 0..4
    strand: np.ndarray  # int32 [N], strand index from 0
    n_strands: int

    @property
    def N(self) -> int:
        return int(self.n3.shape[0])


def _btypes_from_sequence(seq: str) -> List[int]:
    out: List[int] = []
    i = 0
    while i < len(seq):
        c = seq[i]
        if c == "(":
            j = seq.index(")", i)
            out.append(int(seq[i + 1:j]))
            i = j + 1
            continue
        code = BASE_CODE.get(c.upper())
        if code is None:
            raise OxDNAFormatError(f"invalid base {c!r}")
        out.append(code)
        i += 1
    return out


def read_topology(path: str) -> Topology:
    with open(path) as fh:
        lines = [ln.rstrip("\n") for ln in fh]
    header = lines[0].split()
    if len(header) < 2:
        raise OxDNAFormatError("topology header must hold N and the number of strands")
    N, n_strands = int(header[0]), int(header[1])
    n3 = np.full(N, -1, np.int32)
    n5 = np.full(N, -1, np.int32)
    btype = np.zeros(N, np.int32)
    strand = np.zeros(N, np.int32)
    body = [ln for ln in lines[1:] if ln.strip() and not ln.startswith("#")]
    if len(header) >= 3 and header[2] == "5->3":
        idx = 0
        for s, ln in enumerate(body):
            parts = ln.split()
            seq = parts[0]
            circular = any(p.lower() in ("circular=true", "circular=1") for p in parts[1:])
            bts = _btypes_from_sequence(seq)
            first = idx
            for k, bt in enumerate(bts):
                if idx >= N:
                    raise OxDNAFormatError("more nucleotides than the header declares")
                btype[idx] = bt
                strand[idx] = s
                if k > 0:
                    n5[idx] = idx - 1
                if k < len(bts) - 1:
                    n3[idx] = idx + 1
                elif circular:
                    n3[idx] = first
                    n5[first] = idx
                idx += 1
        if idx != N:
            raise OxDNAFormatError(f"header declares {N} nucleotides, strands hold {idx}")
    else:
        if len(body) != N:
            raise OxDNAFormatError(f"header declares {N} nucleotides, file lists {len(body)}")
        for i, ln in enumerate(body):
            parts = ln.split()
            if len(parts) < 4:
                raise OxDNAFormatError(f"line {i + 2} of the topology has an invalid syntax")
            strand[i] = int(parts[0]) - 1
            base = parts[1]
            btype[i] = BASE_CODE[base.upper()] if len(base) == 1 else int(base)
            n3[i] = int(parts[2])
            n5[i] = int(parts[3])
    if len(header) >= 3 and header[2] == "5->3":
        # new layout: type = btype mod 4 for every code (DNAInteraction.cpp:1539)
        typ = np.array([type_from_btype(int(b)) for b in btype], np.int32)
    else:
        # old layout: a single character decodes straight to its type, D included
        # (TopologyParser.cpp:96-109); integer codes map as in the new layout
        typ = np.array([4 if b == 4 else type_from_btype(int(b)) for b in btype], np.int32)
    return Topology(n3, n5, btype, typ, strand, n_strands)


def write_topology(path: str, top: Topology) -> None:
    """Old layout ("strand base n3 n5"), which every reference version reads."""
    with open(path, "w") as fh:
        fh.write(f"{top.N} {top.n_strands}\n")
        for i in range(top.N):
            b = int(top.btype[i])
            base = BASE_CHAR[b] if 0 <= b <= 4 else str(b)
            fh.write(f"{int(top.strand[i]) + 1} {base} {int(top.n3[i])} {int(top.n5[i])}\n")


@dataclasses.dataclass
class Configuration:
    t: int
    box: np.ndarray  # [3]
    pos: np.ndarray  # [N, 3]
    a1: np.ndarray  # [N, 3]
    a3: np.ndarray  # [N, 3]
    vel: np.ndarray  # [N, 3]
    L: np.ndarray  # [N, 3]
    energy: Optional[List[float]] = None


def read_conf(path: str) -> Configuration:
    with open(path) as fh:
        lines = [ln for ln in fh if ln.strip()]
    t = None
    box = None
    energy = None
    k = 0
    while k < len(lines) and re.match(r"^\s*[tbE]\s*=", lines[k]):
        key, val = lines[k].split("=", 1)
        key = key.strip()
        if key == "t":
            t = int(float(val.split()[0]))
        elif key == "b":
            box = np.array([float(x) for x in val.split()[:3]])
        else:
            energy = [float(x) for x in val.split()]
        k += 1
    if box is None:
        raise OxDNAFormatError("configuration without a box line")
    data = np.array([[float(x) for x in ln.split()] for ln in lines[k:]], dtype=np.float64)
    if data.ndim != 2 or data.shape[1] not in (9, 15):
        raise OxDNAFormatError("configuration lines must hold 9 or 15 numbers")
    N = data.shape[0]
    vel = data[:, 9:12] if data.shape[1] == 15 else np.zeros((N, 3))
    L = data[:, 12:15] if data.shape[1] == 15 else np.zeros((N, 3))
    return Configuration(t or 0, box, data[:, 0:3].copy(), data[:, 3:6].copy(), data[:, 6:9].copy(),
                         vel.copy(), L.copy(), energy)


def write_conf(path: str, conf: Configuration) -> None:
    with open(path, "w") as fh:
        fh.write(f"t = {conf.t}\n")
        fh.write("b = %.17g %.17g %.17g\n" % tuple(conf.box))
        e = conf.energy or [0.0, 0.0, 0.0]
        fh.write("E = " + " ".join("%.17g" % x for x in e) + "\n")
        for i in range(conf.pos.shape[0]):
            row = np.concatenate([conf.pos[i], conf.a1[i], conf.a3[i], conf.vel[i], conf.L[i]])
            fh.write(" ".join("%.17g" % x for x in row) + "\n")


def orthonormal_frame(a1: np.ndarray, a3: np.ndarray):
    """The reference's frame clean-up after reading a configuration
    (src/Backends/SimBackend.cpp:622-629): normalise a1 and a3, remove from a1 its a3
    component, renormalise, and a2 = a3 x a1."""
    a1 = a1 / np.linalg.norm(a1, axis=-1, keepdims=True)
    a3 = a3 / np.linalg.norm(a3, axis=-1, keepdims=True)
    a1 = a1 - a3 * np.sum(a1 * a3, axis=-1, keepdims=True)
    a1 = a1 / np.linalg.norm(a1, axis=-1, keepdims=True)
    a2 = np.cross(a3, a1)
    a2 = a2 / np.linalg.norm(a2, axis=-1, keepdims=True)
    return a1, a2, a3


def frame_to_quat(a1: np.ndarray, a2: np.ndarray, a3: np.ndarray) -> np.ndarray:
    """Quaternion (x, y, z, w) of the rotation whose columns are a1, a2, a3 (the inverse of
    src/CUDA/cuda_utils/CUDA_lr_common.cuh:40-61), by Shepperd's method."""
    N = a1.shape[0]
    m = np.stack([a1, a2, a3], axis=-1)  # m[:, i, j] = column j
    q = np.zeros((N, 4))
    tr = m[:, 0, 0] + m[:, 1, 1] + m[:, 2, 2]
    for i in range(N):
        M = m[i]
        t = tr[i]
        if t > 0:
            s = 0.5 / math.sqrt(t + 1.0)
            w = 0.25 / s
            x = (M[2, 1] - M[1, 2]) * s
            y = (M[0, 2] - M[2, 0]) * s
            z = (M[1, 0] - M[0, 1]) * s
        elif M[0, 0] > M[1, 1] and M[0, 0] > M[2, 2]:
            s = 2.0 * math.sqrt(1.0 + M[0, 0] - M[1, 1] - M[2, 2])
            w = (M[2, 1] - M[1, 2]) / s
            x = 0.25 * s
            y = (M[0, 1] + M[1, 0]) / s
            z = (M[0, 2] + M[2, 0]) / s
        elif M[1, 1] > M[2, 2]:
            s = 2.0 * math.sqrt(1.0 + M[1, 1] - M[0, 0] - M[2, 2])
            w = (M[0, 2] - M[2, 0]) / s
            x = (M[0, 1] + M[1, 0]) / s
            y = 0.25 * s
            z = (M[1, 2] + M[2, 1]) / s
        else:
            s = 2.0 * math.sqrt(1.0 + M[2, 2] - M[0, 0] - M[1, 1])
            w = (M[1, 0] - M[0, 1]) / s
            x = (M[0, 2] + M[2, 0]) / s
            y = (M[1, 2] + M[2, 1]) / s
            z = 0.25 * s
        qq = np.array([x, y, z, w])
        q[i] = qq / np.linalg.norm(qq)
    return q


def quat_to_frame(q: np.ndarray):
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    a1 = np.stack([x * x - y * y - z * z + w * w, 2 * (x * y + z * w), 2 * (x * z - y * w)], -1)
    a2 = np.stack([2 * (x * y - z * w), -x * x + y * y - z * z + w * w, 2 * (y * z + x * w)], -1)
    a3 = np.stack([2 * (x * z + y * w), 2 * (y * z - x * w), -x * x - y * y + z * z + w * w], -1)
    return a1, a2, a3


def parse_input(text: str) -> Dict[str, str]:
    """`key = value` lines; '#' starts a comment; `name = { ... }` blocks are kept verbatim."""
    out: Dict[str, str] = {}
    depth = 0
    block_key = None
    block: List[str] = []
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        if depth > 0:
            depth += line.count("{") - line.count("}")
            block.append(line)
            if depth == 0:
                out[block_key] = "\n".join(block)
            continue
        if "=" not in line:
            raise OxDNAFormatError(f"malformed input line {raw!r}")
        key, val = (s.strip() for s in line.split("=", 1))
        if val.startswith("{"):
            depth = val.count("{") - val.count("}")
            block_key = key
            block = [val]
            if depth == 0:
                out[key] = val
            continue
        out[key] = val
    return out


def read_input(path: str) -> Dict[str, str]:
    with open(path) as fh:
        return parse_input(fh.read())


def get_temperature(raw: str) -> float:
    """Simulation units from '300K', '27C' or a bare number (Utils::get_temperature)."""
    m = re.match(r"^\s*([-+0-9.eE]+)\s*([cCkK]?)\s*$", raw)
    if not m:
        raise OxDNAFormatError(f"unrecognizable temperature {raw!r}")
    v = float(m.group(1))
    unit = m.group(2).lower()
    if unit == "c":
        return (v + 273.15) * 0.1 / 300.0
    if unit == "k":
        return v * 0.1 / 300.0
    return v


def read_seq_dep_file(path: str) -> Dict[str, float]:
    return {k: float(v) for k, v in read_input(path).items()}


def parse_bool(v: str) -> bool:
    s = v.strip().lower()
    if s in ("1", "true", "yes", "y"):
        return True
    if s in ("0", "false", "no", "n"):
        return False
    raise OxDNAFormatError(f"not a boolean: {v!r}")
