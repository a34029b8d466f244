"""Reading a function of the reference from its source text, for the golden-vector
scripts beside this file (they run only where the reference's sources are).

The reference's driver is Python 2, so its modules cannot be imported.  A
function is taken from the file as text — from its ``def`` line to the first
code line indented no deeper — and only its Python 2 forms are rewritten:
``print >> f, x`` and ``print x`` become print() calls (trailing comments are
dropped first), ``d.has_key(k)`` becomes ``k in d``, and the caller may add
literal replacements (for a Python 2 integer division).  Nothing else changes.
"""
import os
import re
import sys
import textwrap


def reference_file(name):
    """Path of ``name`` inside the reference's source tree, whose root is given
    by ``--reference DIR`` on the command line or the PYGW_REFERENCE
    environment variable."""
    root = None
    if "--reference" in sys.argv:
        i = sys.argv.index("--reference")
        if i + 1 < len(sys.argv):
            root = sys.argv[i + 1]
    root = root or os.environ.get("PYGW_REFERENCE")
    if not root:
        sys.exit("give the reference's source tree: --reference DIR (or PYGW_REFERENCE=DIR)")
    path = os.path.join(root, name)
    if not os.path.exists(path):
        sys.exit(f"{path} not found")
    return path


class NS:
    """A stand-in object with the given attributes."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def split_comment(line):
    """(code, comment) of a source line: the first # outside a string literal."""
    quote = None
    for i, ch in enumerate(line):
        if quote:
            if ch == quote and line[i - 1] != "\\":
                quote = None
        elif ch in "'\"":
            quote = ch
        elif ch == "#":
            return line[:i].rstrip(), line[i:]
    return line, ""


def py3_line(line, replace=()):
    line, _ = split_comment(line)
    m = re.match(r"^(\s*)print\s*>>\s*(\w+)\s*,\s*(.+)$", line)
    if m:
        line = f"{m.group(1)}print({m.group(3)}, file={m.group(2)})"
    else:
        m = re.match(r"^(\s*)print\s+(?!\()(.+)$", line)
        if m:
            line = f"{m.group(1)}print({m.group(2)})"
    line = re.sub(r"(\w+)\.has_key\(([^()]*)\)", r"(\2 in \1)", line)
    for old, new in replace:
        line = line.replace(old, new)
    return line


def extract(path, head, indent, replace=()):
    """Source of the function whose ``def`` line starts with ``head`` (at
    ``indent``), rewritten for Python 3 and dedented."""
    lines = open(path).read().split("\n")
    start = next(i for i, l in enumerate(lines) if l.startswith(head))
    end = next((i for i in range(start + 1, len(lines))
                if lines[i].strip() and not lines[i].lstrip().startswith("#")
                and not lines[i].startswith(indent + " ")), len(lines))
    return textwrap.dedent("\n".join(py3_line(l, replace) for l in lines[start:end]))


SOURCES = {}        # "path:name" -> source text of each function load() compiled


def load(path, head, indent, namespace, name, replace=()):
    """Compile the extracted function into ``namespace`` and return it."""
    src = extract(path, head, indent, replace)
    SOURCES[f"{path}:{name}"] = src
    exec(compile(src, f"{path}:{name}", "exec"), namespace)
    return namespace[name]


class Trace:
    """Context manager recording which lines of the loaded functions (and of
    Fortran procedures translated by f90py) run."""

    def __init__(self):
        self.hits = {}

    def _global(self, frame, event, arg):
        fn = frame.f_code.co_filename
        return self._local if fn in SOURCES or fn.startswith("<f90:") else None

    def _local(self, frame, event, arg):
        if event == "line":
            self.hits.setdefault(frame.f_code.co_filename, set()).add(frame.f_lineno)
        return self._local

    def __enter__(self):
        sys.settrace(self._global)
        return self

    def __exit__(self, *exc):
        sys.settrace(None)
        return False


def report(trace):
    """Print, per loaded function, how many of its statements ran and those
    that never did."""
    for fn, src in SOURCES.items():
        lines, stack = set(), [compile(src, fn, "exec")]
        while stack:
            c = stack.pop()
            lines.update(ln for _, _, ln in c.co_lines() if ln)
            stack.extend(x for x in c.co_consts if hasattr(x, "co_lines"))
        text = src.split("\n")
        lines = {ln for ln in lines if not text[ln - 1].lstrip().startswith("def ")}
        miss = sorted(lines - trace.hits.get(fn, set()))
        print(f"{fn}: {len(lines) - len(miss)}/{len(lines)} statements executed")
        for ln in miss:
            print("    never:", text[ln - 1].strip())
    f90py = sys.modules.get("f90py")
    hits = {fn[5:-1]: ls for fn, ls in trace.hits.items() if fn.startswith("<f90:")}
    done = set()
    for tr in (f90py.LOADED if f90py else []):      # each translated procedure once
        for unit, (n_run, n_all, miss) in f90py.unexecuted(tr, hits).items():
            if unit in done:
                continue
            done.add(unit)
            print(f"Fortran {unit}: {n_run}/{n_all} statements executed")
            for m in miss:
                print("    never:", m)


def run(main):
    """Run a generator's ``main``; with ``--coverage`` on the command line,
    run it under a Trace with nothing stored and report the statements of the
    reference's functions that no case executed."""
    if "--coverage" not in sys.argv:
        return main()
    import contextlib
    import io
    import numpy as np
    save = np.savez_compressed
    np.savez_compressed = lambda *a, **k: None
    try:
        with Trace() as trace, contextlib.redirect_stdout(io.StringIO()):
            main()
    finally:
        np.savez_compressed = save
    print("(coverage run: nothing stored)")
    report(trace)
