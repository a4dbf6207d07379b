"""ABI check of include/visor_vk.h against the Khronos header the reference vendors.

The ICD must be binary-compatible with applications compiled against the
Khronos Vulkan headers.  This test parses every struct and enum constant of
include/visor_vk.h, compiles a probe that prints sizes, field offsets and enum
values once against our header and once against the reference's
3rdparty/vulkan.h (header version 42), and requires identical output.  It runs
only where the reference tree is present.
"""
import os
import re
import subprocess
import tempfile

import pytest

from conftest import REPO, REFERENCE_DIR

HEADER = os.path.join(REPO, "include", "visor_vk.h")


def _parse_header():
    text = open(HEADER).read()
    structs = []
    for m in re.finditer(r"typedef (struct|union) (\w+) \{(.*?)\} \2;", text, re.S):
        name, body = m.group(2), m.group(3)
        fields = []
        for line in body.split(";"):
            line = line.strip()
            if not line:
                continue
            fm = re.search(r"(\w+)(\[\w+\])?$", line)
            if fm:
                fields.append(fm.group(1))
        structs.append((name, fields))
    enums = re.findall(r"^\s+(VK_[A-Z0-9_]+) = ", text, re.M)
    enums = [e for e in enums if not e.endswith("MAX_ENUM")]
    return structs, enums


def _probe_source(include_line):
    structs, enums = _parse_header()
    lines = ["#include <stdio.h>", "#include <stddef.h>", include_line, "int main(void) {"]
    for name, fields in structs:
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f in fields:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    for e in enums:
        lines.append(f'printf("{e} %lld\\n", (long long){e});')
    lines.append("return 0; }")
    return "\n".join(lines)


def _run(src, incdirs, workdir, tag):
    c = os.path.join(workdir, tag + ".c")
    exe = os.path.join(workdir, tag)
    with open(c, "w") as fh:
        fh.write(src)
    cmd = ["gcc", "-std=c11", "-w", c, "-o", exe] + [f"-I{d}" for d in incdirs]
    subprocess.check_call(cmd)
    return subprocess.check_output([exe]).decode()


@pytest.mark.skipif(not os.path.isdir(REFERENCE_DIR), reason="reference tree not present")
def test_vulkan_header_abi_matches_khronos():
    with tempfile.TemporaryDirectory() as d:
        ours = _run(_probe_source('#include "visor_vk.h"'), [os.path.join(REPO, "include")], d, "ours")
        theirs = _run(
            _probe_source('#include "vulkan.h"'), [os.path.join(REFERENCE_DIR, "3rdparty")], d, "theirs"
        )
    ours_l, theirs_l = ours.splitlines(), theirs.splitlines()
    diffs = [(a, b) for a, b in zip(ours_l, theirs_l) if a != b]
    assert len(ours_l) == len(theirs_l)
    assert not diffs, diffs[:20]
