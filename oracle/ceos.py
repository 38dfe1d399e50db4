"""RADARSAT-1 CEOS raw-data reader restated in numpy, and a writer of the same
layout (test infrastructure only: tests/ and bench.py's CPU legs).

Follows the UBC reader in code/data_process/CEOS:
  * read_CEOS_raw.m:13-16,67-80,108-122: a 16252-byte file header, then
    blocks of 8 range lines; every line is a 192-byte record header, 50 aux
    bytes and 2 x 9288 sample bytes (I, Q); in each block a 2880-byte replica
    sits inside the 7th line, right after its header and aux bytes
    (start_rep = (first_replica - 1) hpa + ha + 1); removing it and reshaping
    the rest as 8 rows of hpa bytes gives the lines;
  * read_CEOS_raw.m:135-141 / load_DATA_block.m:44-46: sample byte d (a 4-bit
    value) decodes to 2 (d - 16 [d > 7]) + 1;
  * extract_AGC.m:45-58: the receiver attenuation is the low 6 bits of aux
    byte 50, d_Rx_AGC - 24 [d_Rx_AGC > 31] dB;
  * load_DATA_block.m:58-69: data *= 1.5 * 10^(AGC_dB / 20) per line (float32).
Sample bytes carry the 4-bit value in the low nibble (what the reader's
'ubit4' path writes and reads back); the decode uses the low nibble.
"""
from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class CeosLayout:
    file_header: int = 16252     # read_CEOS_raw.m:15
    header: int = 192            # per-line record header, :14
    aux: int = 50                # per-line auxiliary bytes, :13
    cells: int = 9288            # range cells per line (tot_Nrg_cells)
    replica: int = 2880          # replica bytes per 8-line block (length_replica)
    replica_line: int = 7        # 1-based line of the block holding the replica (first_replica)
    lines_per_block: int = 8
    agc_byte: int = 50           # 1-based aux byte holding the AGC code (extract_AGC.m:45)
    gain: float = 1.5            # load_DATA_block.m:58

    @property
    def line_bytes(self) -> int:
        return self.header + self.aux + 2 * self.cells

    @property
    def block_bytes(self) -> int:
        return self.replica + self.lines_per_block * self.line_bytes


def decode_nibble(d):
    d = np.asarray(d).astype(np.int16) & 15
    return (2 * (d - 16 * (d > 7)) + 1).astype(np.int16)


def encode_nibble(v):
    """Inverse of decode_nibble for odd values in [-15, 15]."""
    v = np.asarray(v).astype(np.int16)
    return (((v - 1) // 2) & 15).astype(np.uint8)


def agc_db(code):
    d = np.asarray(code).astype(np.int16) & 63
    return (d - 24 * (d > 31)).astype(np.int16)


def line_records(raw: np.ndarray, lay: CeosLayout, first_line: int, nlines: int) -> np.ndarray:
    """[nlines][line_bytes] records of lines first_line.. (0-based), the
    reader's way: whole 8-line blocks, replica removed, reshaped."""
    L8 = lay.lines_per_block
    b0 = first_line // L8
    b1 = (first_line + nlines - 1) // L8 + 1
    rows = []
    start_rep = (lay.replica_line - 1) * lay.line_bytes + lay.header + lay.aux
    for b in range(b0, b1):
        off = lay.file_header + b * lay.block_bytes
        blk = raw[off:off + lay.block_bytes]
        blk = np.concatenate([blk[:start_rep], blk[start_rep + lay.replica:]])
        rows.append(blk.reshape(L8, lay.line_bytes))
    recs = np.concatenate(rows)
    k0 = first_line - b0 * L8
    return recs[k0:k0 + nlines]


def read(raw: np.ndarray, lay: CeosLayout, first_line: int, nlines: int, first_cell: int, ncells: int,
         apply_agc: bool = True):
    """Echo [nlines][ncells] complex64 and AGC attenuation (dB) per line."""
    recs = line_records(np.asarray(raw, dtype=np.uint8), lay, first_line, nlines)
    ha = lay.header + lay.aux
    s = recs[:, ha + 2 * first_cell: ha + 2 * (first_cell + ncells)]
    v = decode_nibble(s).astype(np.float32)
    echo = (v[:, 0::2] + 1j * v[:, 1::2]).astype(np.complex64)
    a = agc_db(recs[:, lay.header + lay.agc_byte - 1])
    if apply_agc:
        g = (np.float32(lay.gain) * (10.0 ** (a.astype(np.float64) / 20.0)).astype(np.float32)).astype(np.float32)
        echo = (echo * g[:, None]).astype(np.complex64)
    return echo, a


def write(samples: np.ndarray, agc_codes: np.ndarray, lay: CeosLayout, first_cell: int = 0, seed: int = 0):
    """CEOS bytes holding `samples` (complex, odd integers in [-15, 15],
    [nlines][ncells]) at cells first_cell.., with per-line AGC codes (low 6
    bits of aux byte agc_byte).  Headers, other aux bytes, the replica and the
    cells outside the sample window are random bytes (the window's nibbles
    are exact)."""
    nlines, ncells = samples.shape
    assert first_cell + ncells <= lay.cells
    rng = np.random.default_rng(seed)
    L8 = lay.lines_per_block
    nblk = (nlines + L8 - 1) // L8
    recs = rng.integers(0, 256, (nblk * L8, lay.line_bytes), dtype=np.uint8)
    ha = lay.header + lay.aux
    recs[:, ha:] &= 15
    recs[:nlines, ha + 2 * first_cell: ha + 2 * (first_cell + ncells): 2] = encode_nibble(samples.real)
    recs[:nlines, ha + 2 * first_cell + 1: ha + 2 * (first_cell + ncells): 2] = encode_nibble(samples.imag)
    j = lay.header + lay.agc_byte - 1
    recs[:nlines, j] = (recs[:nlines, j] & 0xC0) | (np.asarray(agc_codes, dtype=np.uint8) & 63)
    start_rep = (lay.replica_line - 1) * lay.line_bytes + ha
    out = [rng.integers(0, 256, lay.file_header, dtype=np.uint8)]
    for b in range(nblk):
        flat = recs[b * L8:(b + 1) * L8].reshape(-1)
        rep = rng.integers(0, 16, lay.replica, dtype=np.uint8)
        out.append(np.concatenate([flat[:start_rep], rep, flat[start_rep:]]))
    return np.concatenate(out)
