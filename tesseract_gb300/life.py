"""`alpha life --dims D` on the GPU: one Game of Life board over a cube of 2^D machines.

The program is the reference's gen_life_cube (src/gen.c:285-319): a w x h tile in every machine,
2^rbits rows by 2^cbits columns of machines in Gray-code order, edges fetched over links, one
generation per pass.  The board is seeded as cmd_life seeds it (src/work.c:588-592):
splitmix64 from 42, one full 64-bit word per board cell and line word, group by group, so each
cell is Bernoulli(0.5).  The passes run on the GPU cube engine (Cube); this module only maps
between machines and the board.
"""
from __future__ import annotations

import numpy as np

import tesseract_gb300 as T

GOLDEN_GAMMA = np.uint64(0x9E3779B97F4A7C15)


def splitmix64_stream(seed: int, n: int) -> np.ndarray:
    """The first n outputs of splitmix64 from state `seed`, vectorised."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + GOLDEN_GAMMA * np.arange(1, n + 1, dtype=np.uint64)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def gray(x):
    return x ^ (x >> 1)


class LifeCube:
    def __init__(self, dims: int = 16, rbits: int | None = None, w: int = 32, h: int = 32):
        self.rbits = dims // 2 if rbits is None else rbits
        self.cbits = dims - self.rbits
        self.w, self.h = w, h
        self.program = T.Program.gen_life_cube(w, h, self.rbits, self.cbits)
        self.cube = T.Cube(self.program)
        self.machines = self.cube.machines
        self.cells = np.array(self.program.board, dtype=np.int64)  # tile cell i -> cell address
        R = np.arange(1 << self.rbits)[:, None]
        Cc = np.arange(1 << self.cbits)[None, :]
        self.grid = (gray(R) << self.cbits) | gray(Cc)  # tile (R, C) -> machine

    # ---- state ---------------------------------------------------------------------------
    def seed(self, seed: int = 42):
        """cmd_life's random board (src/work.c:588-592) on the device."""
        groups, ncell = self.cube.groups, len(self.cells)
        z = splitmix64_stream(seed, groups * ncell * 8).reshape(groups, ncell, 8)
        mem, rr = self.cube.read()
        words = z.view(np.uint32).reshape(groups, ncell, 16)  # little-endian halves
        for i, c in enumerate(self.cells):
            mem[c] = words[:, i, :].reshape(-1)
        self.cube.write(mem, rr)

    def set_board(self, board: np.ndarray):
        """The whole torus from 0/1 bytes, (2^rbits h) x (2^cbits w), the layout board() reads."""
        nr, nc = 1 << self.rbits, 1 << self.cbits
        t = np.asarray(board, dtype=np.uint8).reshape(nr, self.h, nc, self.w).transpose(1, 3, 0, 2)
        bits = np.zeros((self.h * self.w, self.machines), dtype=np.uint8)
        bits[:, self.grid] = t.reshape(self.h * self.w, nr, nc)
        words = np.packbits(bits, axis=1, bitorder="little").view(np.uint32)
        mem, rr = self.cube.read()
        for i, c in enumerate(self.cells):
            mem[c] = words[i]
        self.cube.write(mem, rr)

    def tile_bits(self):
        """bits[i, m]: tile cell i of machine m."""
        mem, _ = self.cube.read()
        sel = mem[self.cells]  # (cells, W) words
        return np.unpackbits(sel.view(np.uint8), axis=1, bitorder="little")

    def board(self) -> np.ndarray:
        """The whole torus, (2^rbits h) x (2^cbits w), as 0/1 bytes."""
        bits = self.tile_bits()  # (h*w, machines)
        t = bits[:, self.grid]   # (h*w, 2^rb, 2^cb)
        t = t.reshape(self.h, self.w, 1 << self.rbits, 1 << self.cbits)
        return np.ascontiguousarray(t.transpose(2, 0, 3, 1)).reshape(
            (1 << self.rbits) * self.h, (1 << self.cbits) * self.w)

    def run(self, gens: int) -> float:
        """gens generations; returns the device time in ms."""
        return self.cube.run(gens)


def pack_rows(board: np.ndarray) -> np.ndarray:
    """0/1 bytes -> rows of uint64 words (bit j of word k = column 64 k + j)."""
    return np.packbits(board, axis=1, bitorder="little").view(np.uint64).copy()


def unpack_rows(words: np.ndarray) -> np.ndarray:
    return np.unpackbits(words.view(np.uint8), axis=1, bitorder="little")
