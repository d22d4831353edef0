"""The Fortran host shim (fortran/) against the C-ABI, checked as text: no
Fortran compiler exists on the build image or on the GPU machine.

* swm_gpu_c.f90 binds every function that include/swm_gpu.h declares, under
  the same C name, with the same number of arguments;
* stvec_swm_gpu_t overrides every procedure of the reference's stvec_t
  (stvec_mod.f90:13-28), and the operator / time-scheme types override the
  deferred apply / step bindings (operator_mod.f90:11-16, timescheme_mod.f90:
  9-12);
* both files keep to free-form source rules a compiler would enforce first:
  lines of at most 132 characters and balanced program units and blocks.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "swm_gpu.h")
CMOD = os.path.join(ROOT, "fortran", "swm_gpu_c.f90")
SHIM = os.path.join(ROOT, "fortran", "swm_gpu_shim.f90")

# procedures of stvec_t (stvec_mod.f90:13-28)
STVEC_PROCEDURES = {"copy_to", "create_similar", "update_s1v1", "update_s1v1s2v2", "assign_s1",
                    "assign_s1v1", "assign_s1v1s2v2", "algebraic_norm2", "algebraic_dot"}


def _c_prototypes():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    protos = {}
    for m in re.finditer(r"(?:^|\n)\s*(?:const\s+)?(?:int|void|char|size_t)\s*\*?\s*(swm_\w+)\s*\(([^;]*?)\)\s*;",
                         text):
        args = m.group(2).strip()
        n = 0 if args in ("", "void") else len(args.split(","))
        protos[m.group(1)] = n
    return protos


def _fortran_lines(path):
    """Source lines with comments removed and & continuations joined."""
    out, cur = [], ""
    for raw in open(path):
        line = raw.split("!", 1)[0].rstrip() if '"' not in raw.split("!", 1)[0] else raw.rstrip()
        if "!" in line and '"' in line:
            # strip a trailing comment outside the string literals
            q = False
            for k, ch in enumerate(line):
                if ch == '"':
                    q = not q
                elif ch == "!" and not q:
                    line = line[:k].rstrip()
                    break
        if line.endswith("&"):
            cur += line[:-1] + " "
            continue
        cur += line.lstrip() if cur else line
        out.append(cur)
        cur = ""
    return out


def _fortran_bindings():
    binds = {}
    for line in _fortran_lines(CMOD):
        m = re.search(r"(?:function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*bind\(c,\s*name=\"(swm_\w+)\"\)", line)
        if m:
            assert m.group(1) == m.group(3), line
            args = [a for a in m.group(2).split(",") if a.strip()]
            binds[m.group(3)] = len(args)
    return binds


def test_every_header_function_is_bound():
    protos = _c_prototypes()
    binds = _fortran_bindings()
    assert len(protos) > 80
    assert set(protos) == set(binds), (set(protos) ^ set(binds))
    for name, n in protos.items():
        assert binds[name] == n, (name, n, binds[name])


def test_shim_overrides_the_abstract_interfaces():
    src = open(SHIM).read()
    m = re.search(r"type, extends\(stvec_t\) :: stvec_swm_gpu_t(.*?)end type stvec_swm_gpu_t", src, re.S)
    bound = set(re.findall(r"procedure, public :: (\w+)\s*=>", m.group(1)))
    assert STVEC_PROCEDURES <= bound, STVEC_PROCEDURES - bound
    for t, proc in (("operator_swm_gpu_t", "apply"), ("operator_swm_diff_gpu_t", "apply"),
                    ("rk4_gpu_t", "step"), ("explicit_Eul1_gpu_t", "step")):
        m = re.search(r"type, extends\(\w+\) :: %s(.*?)end type %s" % (t, t), src, re.S)
        assert m and re.search(r"procedure, public :: %s\s*=>" % proc, m.group(1)), t
    # every procedure the types bind is defined in the module
    for target in re.findall(r"procedure, public :: \w+\s*=>\s*(\w+)", src):
        assert re.search(r"(?:subroutine|function) %s\(" % target, src), target


def _blocks_balanced(path):
    opens = {"module": 0, "function": 0, "subroutine": 0, "interface": 0, "type": 0, "select": 0,
             "do": 0, "if": 0}
    for line in _fortran_lines(path):
        s = line.strip().lower()
        if not s:
            continue
        if re.match(r"end\s*(module|function|subroutine|interface|type|select|do|if)\b", s):
            kind = re.match(r"end\s*(\w+)", s).group(1)
            opens[kind] -= 1
            assert opens[kind] >= 0, (path, line)
            continue
        if re.match(r"module\s+\w+$", s):
            opens["module"] += 1
        elif re.match(r"(.*\s)?function\s+\w+\s*\(", s) and not s.startswith("procedure"):
            opens["function"] += 1
        elif re.match(r"(recursive\s+)?subroutine\s+\w+", s):
            opens["subroutine"] += 1
        elif s == "interface" or re.match(r"abstract\s+interface$", s):
            opens["interface"] += 1
        elif re.match(r"type\s*(,.*)?::\s*\w+$", s):
            opens["type"] += 1
        elif re.match(r"select\s+type\s*\(", s):
            opens["select"] += 1
        elif re.match(r"(\w+:\s*)?do\s+\w+\s*=", s) or s == "do":
            opens["do"] += 1
        elif re.match(r"(else\s+)?if\s*\(.*\)\s*then$", s):
            if not s.startswith("else"):
                opens["if"] += 1
    return opens


def test_free_form_rules():
    for path in (CMOD, SHIM):
        for k, raw in enumerate(open(path), 1):
            assert len(raw.rstrip("\n")) <= 132, (path, k)
        assert all(v == 0 for v in _blocks_balanced(path).values()), (path, _blocks_balanced(path))
