"""Parsers for the reference's schedule artefacts.

`block_parallel.txt` is the report the reference writes (block.cu:822-925);
`schedule.txt` is what oracle/ref_seam/ref_sgd_dump.cpp writes when the
reference's block_problem hands its schedule to sgd_train.
"""
import gzip


def _open(path):
    return gzip.open(path, "rt") if path.endswith(".gz") else open(path)


def parse_report(path):
    header, blocks, seqs = {}, [], []
    section = None
    with _open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            if line.startswith("# "):
                parts = line[2:].split()
                header[parts[0]] = int(parts[1])
            elif line == "[blocks]":
                section = "blocks"
            elif line == "[parallel_sequences]":
                section = "seqs"
            elif not line or line.startswith("block_id") or line.startswith("sequence_id"):
                continue
            elif section == "blocks":
                p = line.split()
                blocks.append(dict(id=int(p[0]), nnz=int(p[1]), levels=(int(p[2]), int(p[3]), int(p[4])),
                                   ids=(p[5], p[7], p[9]), ranges=(p[6], p[8], p[10])))
            elif section == "seqs":
                p = line.split()
                seqs.append(dict(size=int(p[1]), total_nnz=int(p[2]),
                                 ids=[int(v) for v in p[3].split(",")]))
    return header, blocks, seqs


def parse_schedule(path):
    out = dict(slots=[])
    with _open(path) as f:
        cur = None
        for line in f:
            p = line.split()
            if not p:
                continue
            if p[0] in ("num_parallel", "max_parallel", "scheduled", "train_nnz"):
                out[p[0]] = int(p[1])
            elif p[0] == "num_bs":
                out["num_bs"] = [int(v) for v in p[1:]]
            elif p[0] == "slot":
                cur = dict(id=int(p[2]), nnz=int(p[3]),
                           coe=(float.fromhex(p[4]), float.fromhex(p[5]), float.fromhex(p[6])),
                           xyz=[])
                out["slots"].append(cur)
            else:
                cur["xyz"].append((int(p[0]), int(p[1]), int(p[2])))
    return out
