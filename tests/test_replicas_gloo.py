"""Replica runs (one independent solve per GPU): the host-side aggregation
over ranks, exercised with two gloo ranks on the CPU."""
import os
import socket
import subprocess
import sys
import textwrap

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_rank_throughput_takes_the_slowest_rank(tmp_path):
    script = tmp_path / "worker.py"
    script.write_text(textwrap.dedent("""
        import sys
        sys.path.insert(0, %r)
        from xpfc_cuda_gb300.replicas import Group, throughput
        g = Group("gloo")
        # rank r advanced 1000 * (r + 1) grid points in 2 + r seconds
        v = throughput(1000.0 * (g.rank + 1), 2.0 + g.rank, g)
        g.barrier()
        print("RANK", g.rank, g.world, v, g.max(g.rank + 0.5), flush=True)
        g.close()
    """ % REPO))
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(script)], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (o, e) in zip(procs, outs):
        assert p.returncode == 0, e
    lines = sorted(l for o, _ in outs for l in o.splitlines() if l.startswith("RANK"))
    assert len(lines) == 2
    for line in lines:
        _, rank, world, v, mx = line.split()
        assert world == "2"
        assert abs(float(v) - 3000.0 / 3.0) < 1e-9      # (1000 + 2000) points / slowest 3 s
        assert float(mx) == 1.5


def test_single_process_group_is_a_no_op():
    from xpfc_cuda_gb300.replicas import Group, throughput
    g = Group("gloo")
    assert g.world == 1 and g.max(3.0) == 3.0
    assert throughput(10.0, 2.0, g) == 5.0
