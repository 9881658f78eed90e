"""Input-file helpers shared by the tests."""
import os
import re

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_in(prefix):
    with open(os.path.join(GOLDEN, prefix + ".in")) as f:
        return f.read()


def with_groups(text, extra):
    """Append namelist groups (e.g. "&gb300_list bc_penalty='weighted' /")."""
    return text + "\n" + extra + "\n"


def set_key(text, key, value):
    """Replace `key = ...` inside &problem_list (first occurrence)."""
    pat = re.compile(r"(^\s*%s\s*=\s*)([^,\n/]*)" % re.escape(key), re.M)
    new, n = pat.subn(lambda m: m.group(1) + value, text, count=1)
    assert n == 1, key
    return new


def write(tmp_path, name, text):
    p = os.path.join(str(tmp_path), name)
    with open(p, "w") as f:
        f.write(text)
    return p
