"""One rank of the world-size-2 test of bench.py's replica plumbing (run by
torch.distributed.run from tests/test_dist_cpu.py; gloo on CPU)."""
import json
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
import bench  # noqa: E402


def main():
    d = bench.Dist()
    assert d.ws == 2 and d.rank in (0, 1)
    d.barrier()
    # max over ranks of a per-rank time, sum of per-rank work (the rules the
    # bench applies to its timed region)
    mx = d.reduce(1.5 + d.rank, "MAX")
    sm = d.reduce(10.0 * (d.rank + 1), "SUM")
    out = {"rank": d.rank, "max": mx, "sum": sm}
    d.barrier()
    d.close()
    # one file per rank: the ranks share stdout, where lines can interleave
    with open(os.path.join(sys.argv[1], "rank%d.json" % d.rank), "w") as f:
        json.dump(out, f)


if __name__ == "__main__":
    main()
