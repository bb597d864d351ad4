"""Turns reference GLSL into text that g++ compiles, leaving its arithmetic as written.

Test infrastructure: run by oracle/ref/build_ref.sh in a container that holds
the reference tree, writing only into oracle/_ref/ (git-ignored). Nothing of the
reference is copied into the repository; the generated text is a build
intermediate, like the object files made from it.

Two forms:

    glsl_to_cpp.py compute <shader.comp> <entry> <out>
        A compute shader. Only interface lines change: `#version`, `#extension`
        and the `layout(local_size...) in;` line are dropped; every interface
        block `layout(...) [qualifiers] buffer|uniform Block { members };`
        becomes its members as namespace-scope variables (a runtime-sized array
        `T name[]` becomes `T* name`); `void main()` is renamed to `entry`. Every
        other line is kept byte for byte.

    glsl_to_cpp.py function <file.glsl> <name> <out>
        One function of a GLSL library file: the file's single-line `#define`s
        (its sizes and index macros) and the function's text from its signature
        to the matching closing brace, byte for byte.
"""
import re
import sys

BLOCK = re.compile(
    r"layout\s*\([^)]*\)\s*((?:\w+\s+)*?)(buffer|uniform)\s+(\w+)\s*\{([^}]*)\}\s*;", re.S
)


def _members(body: str) -> str:
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.fullmatch(r"(\w+)\s+(\w+)\s*\[\s*\]", decl)
        if m:  # runtime-sized array: a pointer the harness sets
            out.append(f"static {m.group(1)}* {m.group(2)};")
        else:
            out.append(f"static {decl};")
    return " ".join(out)


def compute(src: str, entry: str) -> str:
    text = src
    text = re.sub(r"^\s*#\s*(version|extension)\b.*$", "", text, flags=re.M)
    text = re.sub(r"layout\s*\(\s*local_size_x[^)]*\)\s*in\s*;", "", text)
    text, nblocks = BLOCK.subn(lambda m: _members(m.group(4)), text)
    text, nmain = re.subn(r"\bvoid\s+main\s*\(\s*\)", f"void {entry}()", text)
    if nmain != 1 or nblocks == 0:
        raise SystemExit(f"glsl_to_cpp: unexpected shader form ({nblocks} blocks, {nmain} main)")
    return text


def function(src: str, name: str) -> str:
    lines = src.splitlines()
    defines = [
        ln for ln in lines
        if re.match(r"\s*#\s*define\s+\w+", ln) and not ln.rstrip().endswith("\\")
        and not re.match(r"\s*#\s*define\s+\w+_GLSL\s*$", ln)
    ]
    m = re.search(r"\bvoid\s+%s\s*\(" % re.escape(name), src)
    if not m:
        raise SystemExit(f"glsl_to_cpp: function {name} not found")
    i = src.index("{", m.end())
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                break
    else:
        raise SystemExit(f"glsl_to_cpp: unbalanced braces in {name}")
    return "\n".join(defines) + "\n\n" + src[m.start():j + 1] + "\n"


def main(argv):
    if len(argv) != 5 or argv[1] not in ("compute", "function"):
        raise SystemExit(__doc__)
    with open(argv[2], encoding="utf-8") as fh:
        src = fh.read()
    out = compute(src, argv[3]) if argv[1] == "compute" else function(src, argv[3])
    with open(argv[4], "w", encoding="utf-8") as fh:
        fh.write(f"// generated by oracle/ref/glsl_to_cpp.py from {argv[2]}\n")
        fh.write(out)


if __name__ == "__main__":
    main(sys.argv)
