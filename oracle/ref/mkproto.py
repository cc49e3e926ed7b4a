"""Generate the C headers that Madagascar's build would generate for the
reference's CPU sources, so those sources compile unchanged.

Madagascar derives a module header from annotations inside the .c file:
lines ending in ``/*^*/`` are copied verbatim (the type section guarded by
``#ifndef _<module>_h``), and every function whose signature is followed by a
``/*< ... >*/`` comment gets a prototype.  This script applies the same rule.
It reads the reference sources where they lie and writes only into the output
directory given on the command line (oracle/_ref/include).

Test infrastructure for the oracle's checker; not product code.
"""
import os
import re
import sys

SIG = re.compile(r"(?ms)^([A-Za-z_][\w \t\*]*?(?:\n[\w \t\*]*?)?\b\w+\s*\([^;{}]*?\))\s*/\*<.*?>\*/")


def header_for(src_path, module):
    text = open(src_path).read()
    guard = "_%s_h" % module
    out = ["#ifndef %s" % guard, "#define %s" % guard, '#include <rsf.h>']
    # type section: the #ifndef _<module>_h ... #endif block, if present
    start = text.find("#ifndef %s" % guard)
    if start >= 0:
        body_start = text.index("\n", start) + 1
        depth, pos = 1, body_start
        for m in re.finditer(r"(?m)^#\s*(if|ifdef|ifndef|endif)\b", text[body_start:]):
            depth += -1 if m.group(1) == "endif" else 1
            if depth == 0:
                pos = body_start + m.start()
                break
        out.append(text[body_start:pos].replace("/*^*/", ""))
    for m in SIG.finditer(text):
        sig = " ".join(m.group(1).split())
        if sig.startswith(("return", "if ", "else")):
            continue
        out.append(sig + ";")
    out.append("#endif")
    return "\n".join(out) + "\n"


def main():
    ref_dir, out_dir = sys.argv[1], sys.argv[2]
    os.makedirs(out_dir, exist_ok=True)
    for module in ("fdutil", "ts_kernel", "omputil", "hash"):
        src = os.path.join(ref_dir, module + ".c")
        hdr = header_for(src, module)
        if module == "ts_kernel":
            # ts_kernel.c guards itself with _TS_KERNEL_H
            hdr = hdr.replace("#define _ts_kernel_h", "#define _ts_kernel_h\n#define _TS_KERNEL_H_PROTO")
        with open(os.path.join(out_dir, module + ".h"), "w") as f:
            f.write(hdr)


if __name__ == "__main__":
    main()
