"""Minimal Fortran namelist reader/writer for madwave3's ``input.dat``.

The Fortran host reads one ``&group ... /`` block per module init routine
(SRC/mod_gridYpara_01y2.f:92-109, mod_pot_01y2.f:62-65,
mod_absorcion_01y2.f:42-43, mod_flux_01y2.f:72-73, mod_colini_01y2.f:36,
main_madwave3.f:110).  This reader accepts what those files contain:
case-insensitive keys, ``!`` comments, ``d``/``D`` exponents, quoted strings,
``.true.``/``.false.``, comma or blank separated ``key=value`` pairs and
single-valued or array (``key(1)=``, ``key=1,2,3``) entries.
"""
import re

_TOKEN = re.compile(r"""'[^']*'|"[^"]*"|[^\s,=]+|=""")


def _strip_comment(line):
    out, quote = [], None
    for ch in line:
        if quote:
            out.append(ch)
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def _value(tok):
    t = tok.strip()
    if t[:1] in "'\"":
        return t[1:-1]
    low = t.lower()
    if low in (".true.", "t", ".t."):
        return True
    if low in (".false.", "f", ".f."):
        return False
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(low.replace("d", "e"))
    except ValueError:
        return t


def parse(text):
    """Return {group_name_lower: {key_lower: value or [values]}}."""
    groups = {}
    lines = [_strip_comment(l) for l in text.splitlines()]
    body = "\n".join(lines)
    for m in re.finditer(r"&(\w+)(.*?)(?:^\s*/|/\s*$|/\s*\n|&end)", body,
                         re.S | re.M | re.I):
        name = m.group(1).lower()
        toks = _TOKEN.findall(m.group(2))
        entries, key, vals = {}, None, []
        i = 0
        while i < len(toks):
            if i + 1 < len(toks) and toks[i + 1] == "=":
                if key is not None:
                    entries[key] = vals[0] if len(vals) == 1 else vals
                key = re.sub(r"\(.*\)", "", toks[i]).lower()
                vals = []
                i += 2
                continue
            vals.append(_value(toks[i]))
            i += 1
        if key is not None:
            entries[key] = vals[0] if len(vals) == 1 else vals
        groups[name] = entries
    return groups


def read(path):
    with open(path) as f:
        return parse(f.read())


def _fmt(v):
    if isinstance(v, bool):
        return ".true." if v else ".false."
    if isinstance(v, str):
        return "'%s'" % v
    if isinstance(v, float):
        return repr(v).replace("e", "d") if "e" in repr(v) else repr(v) + "d0"
    if isinstance(v, (list, tuple)):
        return ",".join(_fmt(x) for x in v)
    return str(v)


def dumps(groups):
    out = []
    for name, entries in groups.items():
        out.append("&%s" % name)
        for k, v in entries.items():
            out.append("  %s=%s" % (k, _fmt(v)))
        out.append("/")
    return "\n".join(out) + "\n"
