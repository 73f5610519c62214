"""Packs the reference's own tree-level test inputs into
tests/golden/tree_golden.tar.gz, so that the tree-cost tests run wherever
the repository goes (the reference tree does not travel).

The files are those its whole-tree cost tests read (test/cost_tests:7-17):
  * test/1.fas .. 13.fas and their fixed trees N.fas.tree, N.fas.1.tree,
    N.fas.2.tree, N.fas.3.tree;
  * the golden costs cc.costs, cc1.costs, cc2.costs, cc3.costs and their
    weightfactor:-1 twins cnc*.costs;
  * polymorphic.ss (static_poly.poy) and cost_tests itself (the expected
    static_poly cost is read from it).
They are copied unchanged; the archive is deterministic (sorted members,
fixed owner and time).

Run where the reference is present:
    python tests/golden/make_tree_golden.py [reference test directory]
"""
import io
import os
import sys
import tarfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "tree_golden.tar.gz")


def members():
    names = []
    for k in range(1, 14):
        names.append("%d.fas" % k)
        names += ["%d.fas.tree" % k] + ["%d.fas.%d.tree" % (k, m) for m in (1, 2, 3)]
    names += ["cc%s.costs" % s for s in ("", "1", "2", "3")]
    names += ["cnc%s.costs" % s for s in ("", "1", "2", "3")]
    names += ["polymorphic.ss", "cost_tests"]
    return sorted(names)


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get(
        "POYD_REFERENCE_TEST", "/root/reference/test")
    buf = io.BytesIO()
    import gzip
    with gzip.GzipFile(fileobj=buf, mode="wb", mtime=0) as gz:
        with tarfile.open(fileobj=gz, mode="w") as tar:
            for name in members():
                data = open(os.path.join(src, name), "rb").read()
                info = tarfile.TarInfo(name)
                info.size = len(data)
                info.mtime = 0
                info.mode = 0o644
                tar.addfile(info, io.BytesIO(data))
    with open(OUT, "wb") as f:
        f.write(buf.getvalue())
    print(OUT, len(buf.getvalue()), "bytes,", len(members()), "files")


if __name__ == "__main__":
    main()
