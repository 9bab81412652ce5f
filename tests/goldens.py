"""Loader for the golden fixtures under tests/golden/ (made by make_golden.py)."""
import gzip
import json
import os

import numpy as np

import refdump

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases():
    return sorted(d for d in os.listdir(GOLDEN) if os.path.isfile(os.path.join(GOLDEN, d, "meta.json")))


class Case:
    def __init__(self, name):
        d = os.path.join(GOLDEN, name)
        self.name = name
        self.dir = d
        with open(os.path.join(d, "meta.json")) as f:
            self.meta = json.load(f)
        with gzip.open(os.path.join(d, "input.txt.gz"), "rt") as f:
            rows = [l.split() for l in f if l.strip()]
        self.input_xyz = np.array([[int(a), int(b), int(c)] for a, b, c, _ in rows], np.int32).reshape(-1, 3)
        self.input_val = np.array([float(v) for *_, v in rows], np.float64)
        with gzip.open(os.path.join(d, "shuffled.txt.gz"), "rt") as f:
            self.shuffled = np.array([[int(v) for v in l.split()] for l in f if l.strip()], np.int32).reshape(-1, 3)
        self.header, self.blocks, self.seqs = refdump.parse_report(os.path.join(d, "block_parallel.txt"))
        self.schedule = refdump.parse_schedule(os.path.join(d, "schedule.txt.gz"))

    @property
    def dims(self):
        return self.meta["I"], self.meta["J"], self.meta["K"]

    def shuffled_values(self):
        """values of the shuffled train order (coordinates are unique)."""
        lut = {tuple(r): v for r, v in zip(self.input_xyz.tolist(), self.input_val.tolist())}
        return np.array([lut[tuple(r)] for r in self.shuffled.tolist()], np.float64)
