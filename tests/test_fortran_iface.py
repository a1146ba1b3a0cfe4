"""The Fortran module (adc_ottawa_gb300/fortran/adcgpu_iface.f90) cannot be
compiled on these machines (no Fortran compiler), so its bind(C) interfaces
are checked against include/adcgpu.h by parsing: every interface names a
declared function, passes the same number of arguments, and passes scalars
by value exactly where the C prototype takes a non-pointer."""
import os
import re

import pytest

from tests.conftest import ROOT


def _c_prototypes():
    src = open(os.path.join(ROOT, "include", "adcgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(adcgpu_\w+)\s*\(([^;{]*?)\)\s*;", src):
        args = [a.strip() for a in m.group(3).split(",") if a.strip() and a.strip() != "void"]
        protos[m.group(2)] = args
    return protos


def _fortran_interfaces():
    src = open(os.path.join(ROOT, "adc_ottawa_gb300", "fortran", "adcgpu_iface.f90")).read()
    src = src.replace("&\n", " ")
    out = {}
    for m in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)(.*?)end function", src,
                         flags=re.S | re.I):
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        body = m.group(4)
        by_value, ptr_value = set(), set()
        for line in body.splitlines():
            if "::" in line and re.search(r"\bvalue\b", line.split("::")[0], flags=re.I):
                names = {re.sub(r"\(.*", "", n).strip() for n in line.split("::")[1].split("!")[0].split(",")}
                by_value |= names
                if re.search(r"type\s*\(\s*c_ptr\s*\)", line.split("::")[0], flags=re.I):
                    ptr_value |= names
        out[m.group(3)] = (args, by_value, ptr_value)
    return out


def test_fortran_interfaces_match_header():
    protos = _c_prototypes()
    ifaces = _fortran_interfaces()
    assert len(ifaces) >= 20
    for name, (args, by_value, ptr_value) in ifaces.items():
        assert name in protos, name
        cargs = protos[name]
        assert len(args) == len(cargs), (name, args, cargs)
        for fa, ca in zip(args, cargs):
            c_is_pointer = "*" in ca or "[" in ca
            # a dummy without VALUE is passed by reference (a C pointer); a
            # type(c_ptr) dummy with VALUE passes the pointer itself
            f_is_pointer = fa not in by_value or fa in ptr_value
            assert f_is_pointer == c_is_pointer, (name, fa, ca)
