"""Malformed JAMS config texts: the config front end (llg_config.cu) must
answer every input with a status code, never by crashing, hanging or
writing past the output buffer.  Seeded mutations (truncations, deleted,
repeated and replaced spans, stray grammar characters) of the configs in
jams_gb300.configs go through llg_config_describe, with and without a
patch.  The loop runs in a child process so that a crash fails the test
instead of ending the session; no GPU is needed."""
import ast
import os
import subprocess
import sys
import textwrap

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = textwrap.dedent(r'''
    import ctypes, random, sys
    sys.path.insert(0, ROOT)
    from jams_gb300 import configs as C, llg

    L = llg.lib()
    bases = [C.sc_ferromagnet(L=6, T=10.0, steps=10),
             C.bcc_three_shell(L=5, T=300.0, steps=10),
             C.bcc_three_shell(L=6, T=0.0, steps=10, dipole_cutoff=2.0),
             C.triangular_dmi(L=8, T=5.0, Bz=1.0, steps=10)]
    alphabet = '{}()[];:=",.-+0123456789eE/*#\n\t abcdefghijklmnopqrstuvwxyz_'
    rng = random.Random(20261204)

    def mutate(t):
        for _ in range(rng.randint(1, 4)):
            if not t:
                break
            i = rng.randrange(len(t))
            k = rng.randint(1, 12)
            op = rng.randrange(5)
            if op == 0:
                t = t[:i]
            elif op == 1:
                t = t[:i] + t[i + k:]
            elif op == 2:
                t = t[:i] + t[i:i + k] * rng.randint(2, 4) + t[i:]
            elif op == 3:
                t = t[:i] + rng.choice(alphabet) + t[i + 1:]
            else:
                t = t[:i] + ''.join(rng.choice(alphabet) for _ in range(k)) + t[i:]
        return t

    n = 1 << 20
    guard = 4096
    counts = {}
    for it in range(N):
        base = bases[it % len(bases)]
        text = mutate(base)
        patch = mutate('physics : { temperature = 50.0; };') if it % 5 == 0 else ''
        buf = ctypes.create_string_buffer(n + guard)
        ctypes.memset(ctypes.addressof(buf) + n, 0x5A, guard)
        rc = L.llg_config_describe(text.encode(), patch.encode(), buf, n)
        tail = ctypes.string_at(ctypes.addressof(buf) + n, guard)
        assert tail == b'\x5a' * guard, 'wrote past the buffer'
        if rc != 0:
            msg = L.llg_last_error(None)
            assert msg, 'error without a message'
        counts[rc] = counts.get(rc, 0) + 1
    print('codes', sorted(counts.items()))
''')


def test_mutated_configs_are_answered_with_a_status():
    code = "ROOT = %r\nN = 20000\n" % ROOT + CHILD
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, (res.returncode, res.stdout[-2000:], res.stderr[-4000:])
    codes = dict(ast.literal_eval(res.stdout.strip().split("codes ", 1)[1]))
    assert codes.get(-1, 0) > 0      # most mutations are rejected as bad input
    assert sum(codes.values()) == 20000
