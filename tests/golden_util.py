"""Access to the committed golden fixtures (tests/golden/, made by
tests/golden/make_golden.py from the reference itself)."""
import json
import lzma
import os

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases():
    return json.load(open(os.path.join(GOLDEN, "cases.json")))


def reflog(name):
    """(checksums, cell_hashes, meshes) from the reference's hook log:
    checksums[i] = (var, value) of the i-th check_sum call, cell_hashes[i]
    the hash of that variable's cells, meshes = [(ts, n_active, hash)]."""
    sums, hashes, meshes = [], [], []
    with lzma.open(os.path.join(GOLDEN, name + ".reflog.xz"), "rt") as f:
        for line in f:
            p = line.split()
            if p[0] == "cs":
                v = int(p[3], 16)
                sums.append((int(p[2]),
                             __import__("struct").unpack(
                                 "<d", v.to_bytes(8, "little"))[0]))
                hashes.append(int(p[4], 16))
            elif p[0] == "mesh":
                meshes.append((int(p[1]), int(p[2]), p[3]))
    return sums, hashes, meshes


def trace_path(name):
    return os.path.join(GOLDEN, name + ".trace.xz")


def arg(args, flag, default=None):
    return args[args.index(flag) + 1] if flag in args else default


# Cases too large to replay through the CPU oracle inside the CPU suite;
# they are pinned by make_golden.py (hybrid == reference) and replayed on
# the GPU.
HEAVY = {"config2", "config5"}


def hashed_stages(hashes, V):
    """Checksum stages whose cell hashes the log carries (0 = not taken);
    returns first, middle and last of them."""
    st = [s for s in range(len(hashes) // V) if hashes[s * V] != 0]
    return {st[0], st[len(st) // 2], st[-1]} if st else set()


def mark_cases():
    """Cases with a marking fixture (<name>.mark.xz)."""
    return sorted(f[:-len(".mark.xz")] for f in os.listdir(GOLDEN)
                  if f.endswith(".mark.xz"))


def mark_path(name):
    return os.path.join(GOLDEN, name + ".mark.xz")
