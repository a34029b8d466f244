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


def load(path, head, indent, namespace, name, replace=()):
    """Compile the extracted function into ``namespace`` and return it."""
    exec(compile(extract(path, head, indent, replace), f"{path}:{name}", "exec"), namespace)
    return namespace[name]
