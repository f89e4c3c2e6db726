"""Regenerate tests/golden/examples.json from the reference's example programs.

Reads the OpenQASM 2 files in the reference checkout's examples/ directory
(bell, ghz, qft, grover, teleport, bernstein_vazirani), lowers them with a
small reader for the subset they use (qreg/creg, broadcast, gate macros,
`measure a -> b`, `if (creg == v)`), and stores each as an instruction list
together with the expected output its header comment states. The tests
replay these lists through the oracle and the CUDA backend; nothing at test
time reads the reference checkout.

Usage: python tests/golden/make_golden.py /path/to/zeno/checkout
       (or set ZENO_REFERENCE to the checkout)
"""

import json
import math
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

# Known answers stated in each example's header comment.
EXPECTED = {
    "bell": {"keys": ["00", "11"], "kind": "support"},
    "ghz": {"keys": ["0" * 24, "1" * 24], "kind": "support"},
    "qft": {"keys": ["10110001"], "kind": "exact"},
    "bernstein_vazirani": {"keys": ["110101"], "kind": "exact"},
    "grover": {"keys": ["101"], "kind": "dominant", "p": 0.945},
    "teleport": {"keys": ["1 0 0", "1 0 1", "1 1 0", "1 1 1"], "kind": "support"},
}


def strip_comments(src):
    return re.sub(r"//[^\n]*", "", src)


def parse(src):
    src = strip_comments(src)
    qregs, cregs, gates, instrs = [], [], {}, []
    # gate macros: gate name args { body }
    for m in re.finditer(r"gate\s+(\w+)\s*([^{]*)\{([^}]*)\}", src):
        name, args, body = m.group(1), m.group(2), m.group(3)
        params = []
        am = re.match(r"\(([^)]*)\)\s*(.*)", args.strip())
        if am:
            params = [p.strip() for p in am.group(1).split(",") if p.strip()]
            args = am.group(2)
        gates[name] = (params, [a.strip() for a in args.split(",") if a.strip()],
                       [s.strip() for s in body.split(";") if s.strip()])
    src = re.sub(r"gate\s+\w+[^{]*\{[^}]*\}", "", src)
    stmts = [s.strip() for s in src.split(";") if s.strip()]

    def qoff(name):
        off = 0
        for n, s in qregs:
            if n == name:
                return off, s
            off += s
        raise KeyError(name)

    def coff(name):
        off = 0
        for i, (n, s) in enumerate(cregs):
            if n == name:
                return i, off, s
            off += s
        raise KeyError(name)

    def qarg(a):
        m = re.match(r"(\w+)\s*\[(\d+)\]", a)
        if m:
            o, _ = qoff(m.group(1))
            return [o + int(m.group(2))]
        o, s = qoff(a)
        return [o + i for i in range(s)]

    def emit_gate(name, params, qargs, cond):
        if name in gates:
            fparams, fargs, body = gates[name]
            env = dict(zip(fparams, params))
            amap = dict(zip(fargs, qargs))
            for st in body:
                m = re.match(r"(\w+)\s*(\(([^)]*)\))?\s*(.*)", st)
                sub_params = []
                if m.group(3):
                    sub_params = [eval(p, {"pi": math.pi, **env}) for p in m.group(3).split(",")]
                sub_q = [amap[a.strip()] for a in m.group(4).split(",")]
                emit_gate(m.group(1), sub_params, sub_q, cond)
            return
        instrs.append({"kind": 0, "name": name, "qubits": list(qargs), "params": list(params),
                       "cond": cond})

    for st in stmts:
        if st.startswith("OPENQASM") or st.startswith("include"):
            continue
        m = re.match(r"qreg\s+(\w+)\s*\[(\d+)\]", st)
        if m:
            qregs.append((m.group(1), int(m.group(2))))
            continue
        m = re.match(r"creg\s+(\w+)\s*\[(\d+)\]", st)
        if m:
            cregs.append((m.group(1), int(m.group(2))))
            continue
        cond = None
        m = re.match(r"if\s*\(\s*(\w+)\s*==\s*(\d+)\s*\)\s*(.*)", st, re.S)
        if m:
            ci, _, _ = coff(m.group(1))
            cond = [ci, int(m.group(2))]
            st = m.group(3).strip()
        m = re.match(r"measure\s+(.+?)\s*->\s*(.+)", st)
        if m:
            qs = qarg(m.group(1).strip())
            cm = re.match(r"(\w+)\s*\[(\d+)\]", m.group(2).strip())
            if cm:
                _, o, _ = coff(cm.group(1))
                cls = [o + int(cm.group(2))]
            else:
                _, o, s = coff(m.group(2).strip())
                cls = [o + i for i in range(s)]
            for q, c in zip(qs, cls):
                instrs.append({"kind": 1, "qubits": [q], "clbit": c, "cond": cond})
            continue
        m = re.match(r"reset\s+(.+)", st)
        if m:
            for q in qarg(m.group(1).strip()):
                instrs.append({"kind": 2, "qubits": [q], "cond": cond})
            continue
        if st.startswith("barrier"):
            instrs.append({"kind": 3, "qubits": [], "cond": None})
            continue
        m = re.match(r"(\w+)\s*(\(([^)]*)\))?\s*(.*)", st, re.S)
        name = m.group(1)
        params = [eval(p, {"pi": math.pi}) for p in m.group(3).split(",")] if m.group(3) else []
        args = [qarg(a.strip()) for a in m.group(4).split(",")]
        width = max(len(a) for a in args)
        for i in range(width):  # broadcast over whole registers
            emit_gate(name, params, [a[i] if len(a) > 1 else a[0] for a in args], cond)
    return {"n_qubits": sum(s for _, s in qregs), "cregs": cregs, "instrs": instrs}


def build(ref):
    """The fixture contents for the examples in the checkout at `ref`."""
    out = {}
    for name in sorted(EXPECTED):
        with open(os.path.join(ref, "examples", name + ".qasm")) as f:
            prog = parse(f.read())
        prog["expected"] = EXPECTED[name]
        out[name] = prog
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ZENO_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py /path/to/zeno/checkout (or set ZENO_REFERENCE)")
    out = build(ref)
    with open(os.path.join(HERE, "examples.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "examples.json"), "with", len(out), "programs")


if __name__ == "__main__":
    main()
