"""Reader for the reference's Fortran namelist input files.

The reference reads `&input` and `&param` groups with list-directed namelist
I/O (main.f90:45-51, 137-147).  This reader accepts the subset those files use:
`key = value` entries separated by newlines or commas, values that are
integers, reals with d/D/e exponents, quoted strings, logicals (.true./.false.,
T/F) or whitespace/comma-separated arrays, `!` comments, and a closing `&end`
or `/`.  Keys are returned lower-case.
"""
import re

_LOGICAL = {".true.": True, ".false.": False, "t": True, "f": False, ".t.": True, ".f.": False}


def _value(tok):
    t = tok.strip()
    if not t:
        return None
    if t[0] in "'\"":
        return t[1:-1] if len(t) >= 2 and t[-1] == t[0] else t[1:]
    low = t.lower()
    if low in _LOGICAL:
        return _LOGICAL[low]
    num = low.replace("d", "e")
    try:
        if re.fullmatch(r"[+-]?\d+", num):
            return int(num)
        return float(num)
    except ValueError:
        return t


def _split_values(text):
    out, cur, quote = [], "", None
    for ch in text:
        if quote:
            cur += ch
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
            cur += ch
        elif ch in " \t,":
            if cur:
                out.append(cur)
                cur = ""
        else:
            cur += ch
    if cur:
        out.append(cur)
    return out


def parse(text, group=None):
    """Parse one namelist group from `text`; returns {key: value or list}."""
    lines = []
    for line in text.splitlines():
        # strip comments outside quotes
        q, buf = None, ""
        for ch in line:
            if q:
                buf += ch
                if ch == q:
                    q = None
            elif ch in "'\"":
                q = ch
                buf += ch
            elif ch == "!":
                break
            else:
                buf += ch
        lines.append(buf)
    body = "\n".join(lines)
    m = re.search(r"&(\w+)(.*?)(?:&end|/\s*$|\Z)", body, flags=re.S | re.I)
    if not m:
        raise ValueError("no namelist group found")
    if group is not None and m.group(1).lower() != group.lower():
        raise ValueError(f"expected group {group}, found {m.group(1)}")
    content = m.group(2)
    parts = re.split(r"(\b[A-Za-z_]\w*(?:\(\d+\))?\s*=)", content)
    result = {}
    for i in range(1, len(parts) - 1, 2):
        key = parts[i].rstrip("=").strip().lower()
        vals = [_value(v) for v in _split_values(parts[i + 1].replace("\n", " "))]
        vals = [v for v in vals if v is not None]
        result[key] = vals[0] if len(vals) == 1 else vals
    return result


def read(path, group=None):
    with open(path) as f:
        return parse(f.read(), group)
