"""The reference's golden-file comparison rule, restated for the parity tests.

TestUtils.compareFilesWithUnOrderedFields (genomix-data/.../utils/TestUtils.java:67-136)
with compareGeneLettersByFields (:138-181), as BatchTestFilesTest calls it with
tobeSorted=true and unordered fields {1, 2, 3, 4} (BatchTestFilesTest.java:171-172).
"""
import functools
import re

_NON_GENE = re.compile(r"[^ATCG]+")


def _java_split(s: str, pattern: str):
    """String.split(regex): trailing empty strings are removed."""
    parts = re.split(pattern, s)
    if len(parts) == 1:
        return parts
    while parts and parts[-1] == "":
        parts.pop()
    return parts


def _field_cmp(unordered):
    def cmp(a, b):
        if not unordered:
            return (a > b) - (a < b)
        pa, pb = _java_split(a, "\t"), _java_split(b, "\t")
        for i in range(len(pa)):
            if i in unordered:
                continue
            x, y = pa[i], pb[i] if i < len(pb) else ""
            if x != y:
                return (x > y) - (x < y)
        return 0
    return cmp


def _gene_fields_equal(exp: str, act: str, unordered) -> bool:
    if exp == act:
        return True
    fe, fa = _java_split(exp, "\t"), _java_split(act, "\t")
    if len(fa) != len(fe):
        return False
    ue, ua = [], []
    for i in range(len(fa)):
        if i in unordered:
            ue.append(fe[i])
            ua.append(fa[i])
        elif fa[i] != fe[i]:
            return False
    for a, e in zip(ua, ue):
        sa = sorted(_java_split(a, "[^ATCG]+"))
        se = sorted(_java_split(e, "[^ATCG]+"))
        for j in range(len(sa)):
            if j >= len(se) or sa[j] != se[j]:
                return False
    return True


def compare_unordered(expected_text: str, actual_text: str, unordered=frozenset({1, 2, 3, 4})):
    """Raises AssertionError where the reference's test would throw."""
    act = [l for l in actual_text.splitlines()]
    exp = [l for l in expected_text.splitlines()]
    key = functools.cmp_to_key(_field_cmp(unordered))
    act.sort(key=key)
    exp.sort(key=key)
    for n, a in enumerate(act):
        assert n < len(exp), f"actual has more lines than expected at line {n + 1}: {a}"
        assert _gene_fields_equal(exp[n], a, unordered), f"line {n + 1} differs:\n< {exp[n]}\n> {a}"
    assert len(act) >= len(exp), "expected file has more lines"


def strict_normal_form(text: str):
    """A stricter form than the reference's: every line, with the four edge lists sorted."""
    out = []
    for line in text.splitlines():
        f = line.split("\t")
        for i in (1, 2, 3, 4):
            name, _, lst = f[i].partition(":")
            if lst.startswith("[") and lst.endswith("]") and lst != "[]":
                lst = "[" + ",".join(sorted(lst[1:-1].split(","))) + "]"
            f[i] = name + ":" + lst
        out.append("\t".join(f))
    return sorted(out)
