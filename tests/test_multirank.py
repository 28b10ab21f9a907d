"""Multi-process host logic of the benchmark on CPU (gloo, world size 2):
every rank advances its own tile block (weak scaling, no data-path
collective) and the timed region is reduced with MAX over ranks."""
import os
import socket
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_max_reduction_and_disjoint_shards(tmp_path):
    script = tmp_path / "w.py"
    script.write_text(textwrap.dedent("""
        import os, sys, json
        sys.path.insert(0, %r)
        import bench
        d = bench.Dist(2)
        t = [1.5, 4.0][d.rank]
        m = d.max(t)
        ts = bench.workload(type("A", (), {"mp": 64, "workload": "grid", "steps": 1})(), d.rank)
        print(json.dumps({"rank": d.rank, "max": m, "off": bench.shard_offset(d.rank, 64),
                          "first": int(ts.iveg[0]), "seed": ts.seed}))
        d.close()
    """ % ROOT))
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()), WORLD_SIZE="2")
    procs = []
    for r in range(2):
        e = dict(env, RANK=str(r), LOCAL_RANK=str(r))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=e, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        o, err = p.communicate(timeout=240)
        assert p.returncode == 0, err
        outs.append(__import__("json").loads(o.strip().splitlines()[-1]))
    assert all(o["max"] == 4.0 for o in outs)
    assert outs[0]["off"] == 0 and outs[1]["off"] == 64
    assert outs[0]["seed"] != outs[1]["seed"]
