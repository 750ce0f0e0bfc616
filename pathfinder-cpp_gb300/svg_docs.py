"""Synthetic SVG documents: a few written by hand, and a seeded generator (tests and bench).

The generator draws every element and attribute form the parser handles (shapes, path data
with all commands in absolute and relative form and the compact number syntax, nested groups
with transforms, presentation attributes and style declarations, colour syntaxes, units,
stroke styles, dash arrays, gradients with stop inheritance, view boxes and aspect ratios).
Documents stay within what the reference's parser defines: every transform has its arguments.
"""
from __future__ import annotations

import numpy as np

HAND = {
    "svg_shapes": """<svg xmlns="http://www.w3.org/2000/svg" width="200" height="150" viewBox="0 0 100 75">
<rect x="10" y="10" width="30" height="20" fill="#f80" stroke="navy" stroke-width="2"/>
<circle cx="60" cy="40" r="15" fill="rgb(20, 200, 40)" fill-opacity="0.5"/>
<ellipse cx="30" cy="55" rx="20" ry="8" style="fill:#0af; stroke: red; stroke-width: 1.5; stroke-dasharray: 4 2"/>
<line x1="5" y1="70" x2="95" y2="5" stroke="black" stroke-linecap="round"/>
<polyline points="10,60 20,70 30,60 40,70" fill="none" stroke="purple" stroke-linejoin="bevel" stroke-width="3"/>
<polygon points="70,10 90,30 80,50 60,30" fill="yellow" fill-rule="evenodd" stroke="#123" stroke-linejoin="round"/>
<rect x="50" y="55" width="40" height="15" rx="5" fill="teal"/>
</svg>""",
    "svg_paths": """<svg width="300" height="300">
<g transform="translate(10,20) rotate(15) scale(1.5)">
<path d="M10 10 L50 10 l0 40 h-20 v-10 H10 Z M60 60 C70 40 90 40 100 60 S 120 80 130 60 Q140 40 150 60 T170 60 z"
 fill="#c33" stroke="#333" stroke-width="2" stroke-miterlimit="2"/>
<path d="M20 120 A30 20 0 0 1 80 120 a 20 20 0 1 0 40 0" fill="none" stroke="blue" stroke-width="4" stroke-linecap="square"/>
<path d="m150,150 50,0 0,50 -50,0z m10,10 30,0 0,30 -30,0z" fill="green" fill-rule="evenodd"/>
</g>
<path d="M1e1,2.5e2 l.5.5 -3-4 1.5E1 0" stroke="red" fill="none" transform="matrix(1 0.2 -0.1 1 5 5) skewX(10)"/>
</svg>""",
    "svg_gradients": """<svg width="256" height="256">
<defs>
<linearGradient id="lg" x1="0" y1="0" x2="1" y2="1"><stop offset="0" stop-color="#f00"/>
<stop offset="0.5" stop-color="#0f0" stop-opacity="0.5"/><stop offset="1" stop-color="blue"/></linearGradient>
<radialGradient id="rg" cx="0.5" cy="0.5" r="0.5" spreadMethod="repeat"><stop offset="0%" stop-color="white"/>
<stop offset="100%" stop-color="black"/></radialGradient>
<linearGradient id="lg2" xlink:href="#lg" gradientUnits="userSpaceOnUse" x1="10" y1="10" x2="200" y2="50"
 gradientTransform="rotate(20)"/>
</defs>
<rect x="10" y="10" width="100" height="100" fill="url(#lg)" stroke="url(#rg)" stroke-width="6"/>
<circle cx="180" cy="70" r="50" fill="url(#rg)"/>
<rect x="20" y="150" width="200" height="80" fill="url(#lg2)" transform="scale(1.1 0.9)"/>
<rect x="0" y="0" width="5" height="5" fill="url(#missing)" stroke="none"/>
</svg>""",
    "svg_no_size": """<svg><path d="M-20 -10 C 40 -60 90 80 140 30" stroke="black" stroke-width="3" fill="none"
 stroke-dasharray="5,3,1" stroke-dashoffset="2"/>
<rect x="0" y="0" width="10" height="10" fill="red" opacity="0.5" display="none"/></svg>""",
    "svg_empty": """<?xml version="1.0"?><!-- nothing to draw --><svg width="64" height="32"></svg>""",
    # attributes of the other gradient kind land in the shared coordinate slots (x1/cx, y1/cy,
    # x2/r, y2/fx), and a gradient without stops leaves its shape unpainted
    "svg_gradient_slots": """<svg width="100" height="100"><defs>
<linearGradient id="a" cx="0.2" r="0.9"><stop offset="0" stop-color="red"/><stop offset="1" stop-color="blue"/></linearGradient>
<radialGradient id="b" x1="0.2" x2="0.7" y2="0.4" fy="0.1"><stop offset="0" stop-color="red"/><stop offset="1" stop-color="#0f08"/></radialGradient>
<linearGradient id="c"/></defs>
<rect width="50" height="50" fill="url(#a)"/><circle cx="70" cy="70" r="25" fill="url(#b)" stroke="url(#c)"/></svg>""",
}

_NAMED = ["red", "green", "blue", "yellow", "cyan", "magenta", "black", "grey", "gray", "white", "navy", "olive"]


def _num(rng, lo, hi, compact=False):
    v = rng.uniform(lo, hi)
    k = rng.integers(0, 6)
    if k == 0:
        s = f"{int(round(v))}"
    elif k == 1:
        s = f"{v:.1f}"
    elif k == 2:
        s = f"{v:.3f}"
    elif k == 3:
        s = f"{v:.2e}"
    elif k == 4:
        s = f"{v:.4g}"
    else:
        s = f"{v:.2f}"
    if compact and s.startswith("0.") and rng.random() < 0.5:
        s = s[1:]
    elif compact and s.startswith("-0.") and rng.random() < 0.5:
        s = "-" + s[2:]
    return s


def _color(rng):
    k = rng.integers(0, 6)
    if k == 0:
        return "#" + "".join(f"{c:02x}" for c in rng.integers(0, 256, 3))
    if k == 1:
        return "#" + "".join(f"{c:x}" for c in rng.integers(0, 16, 3))
    if k == 2:
        r, g, b = rng.integers(0, 256, 3)
        return f"rgb({r}, {g}, {b})"
    if k == 3:
        r, g, b = rng.uniform(0, 100, 3)
        return f"rgb({r:.1f}%, {g:.0f}%, {b:.2f}%)"
    return _NAMED[rng.integers(0, len(_NAMED))]


def _transform(rng):
    items = []
    for _ in range(rng.integers(1, 3)):
        k = rng.integers(0, 7)
        if k == 0:
            items.append(f"translate({_num(rng, -40, 40)},{_num(rng, -40, 40)})")
        elif k == 1:
            items.append(f"translate({_num(rng, -40, 40)})")
        elif k == 2:
            items.append(f"rotate({_num(rng, -180, 180)})")
        elif k == 3:
            items.append(f"rotate({_num(rng, -90, 90)} {_num(rng, 0, 200)} {_num(rng, 0, 200)})")
        elif k == 4:
            items.append(f"scale({_num(rng, 0.5, 1.6)}{' ' + _num(rng, 0.5, 1.6) if rng.random() < 0.5 else ''})")
        elif k == 5:
            items.append(f"{'skewX' if rng.random() < 0.5 else 'skewY'}({_num(rng, -30, 30)})")
        else:
            a, d = rng.uniform(0.6, 1.4, 2)
            b, c = rng.uniform(-0.3, 0.3, 2)
            e, f = rng.uniform(-30, 30, 2)
            items.append(f"matrix({a:.3f} {b:.3f} {c:.3f} {d:.3f} {e:.2f} {f:.2f})")
    return " ".join(items)


def _path_data(rng, side):
    parts = [f"M{_num(rng, 0, side)} {_num(rng, 0, side)}"]
    for _ in range(rng.integers(2, 12)):
        cmd = "LHVCSQTAZlhvcsqtaz"[rng.integers(0, 18)]
        rel = cmd.islower()
        lo, hi = (-side / 4, side / 4) if rel else (0, side)
        n = {"l": 2, "h": 1, "v": 1, "c": 6, "s": 4, "q": 4, "t": 2, "a": 0, "z": 0}[cmd.lower()]
        reps = rng.integers(1, 3)
        if cmd in "Zz":
            parts.append(cmd)
            if rng.random() < 0.5:
                parts.append(f"M{_num(rng, 0, side)},{_num(rng, 0, side)}")
            continue
        args = []
        for _ in range(reps):
            if cmd in "Aa":
                args += [_num(rng, 1, side / 3), _num(rng, 1, side / 3), _num(rng, -90, 90),
                         str(rng.integers(0, 2)), str(rng.integers(0, 2)),
                         _num(rng, lo, hi, True), _num(rng, lo, hi, True)]
            else:
                args += [_num(rng, lo, hi, True) for _ in range(n)]
        sep = "," if rng.random() < 0.3 else " "
        parts.append(cmd + sep.join(args))
    return (" " if rng.random() < 0.5 else "").join(parts)


def _style(rng, grads):
    """Fill / stroke attributes, as presentation attributes or one style declaration."""
    decl = {}
    k = rng.random()
    if k < 0.12:
        decl["fill"] = "none"
    elif k < 0.25 and grads:
        decl["fill"] = f"url(#{grads[rng.integers(0, len(grads))]})"
    elif k < 0.85:
        decl["fill"] = _color(rng)
    if rng.random() < 0.3:
        decl["fill-opacity"] = f"{rng.uniform(0, 1):.2f}"
    if rng.random() < 0.2:
        decl["fill-rule"] = "evenodd" if rng.random() < 0.6 else "nonzero"
    if rng.random() < 0.55:
        decl["stroke"] = (f"url(#{grads[rng.integers(0, len(grads))]})" if grads and rng.random() < 0.15
                          else _color(rng))
        unit = ["", "", "px", "pt", "mm", "%", "em"][rng.integers(0, 7)]
        decl["stroke-width"] = _num(rng, 0.3, 6) + unit
        if rng.random() < 0.5:
            decl["stroke-linecap"] = ["butt", "round", "square"][rng.integers(0, 3)]
        if rng.random() < 0.5:
            decl["stroke-linejoin"] = ["miter", "round", "bevel"][rng.integers(0, 3)]
        if rng.random() < 0.3:
            decl["stroke-miterlimit"] = _num(rng, 1, 10)
        if rng.random() < 0.3:
            decl["stroke-opacity"] = f"{rng.uniform(0, 1):.2f}"
        if rng.random() < 0.3:
            k = rng.random()
            if k < 0.1:
                decl["stroke-dasharray"] = "none"
            elif k < 0.15:
                decl["stroke-dasharray"] = "0 0"
            else:
                decl["stroke-dasharray"] = ("," if rng.random() < 0.5 else " ").join(
                    _num(rng, 1, 12) for _ in range(rng.integers(1, 5)))
            if rng.random() < 0.5:
                decl["stroke-dashoffset"] = _num(rng, -5, 5)
    if rng.random() < 0.5:
        return " ".join(f'{k}="{v}"' for k, v in decl.items())
    return 'style="' + "; ".join(f"{k}:{v}" for k, v in decl.items()) + '"'


def _gradients(rng):
    defs, ids = [], []
    for i in range(rng.integers(0, 4)):
        gid = f"g{i}"
        radial = rng.random() < 0.5
        attrs = [f'id="{gid}"']
        if rng.random() < 0.3:
            attrs.append('gradientUnits="userSpaceOnUse"')
            big = True
        else:
            big = False
        span = 200 if big else 1
        if radial:
            for a in ("cx", "cy", "r"):
                if rng.random() < 0.7:
                    attrs.append(f'{a}="{_num(rng, 0.1 * span, span)}"')
            if rng.random() < 0.3:
                attrs.append(f'fx="{_num(rng, 0, span)}" fy="{_num(rng, 0, span)}"')
        else:
            for a in ("x1", "y1", "x2", "y2"):
                if rng.random() < 0.7:
                    attrs.append(f'{a}="{_num(rng, 0, span)}"' if rng.random() < 0.7
                                 else f'{a}="{rng.integers(0, 101)}%"')
        if rng.random() < 0.3:
            attrs.append(f'spreadMethod="{["pad", "reflect", "repeat"][rng.integers(0, 3)]}"')
        if rng.random() < 0.3:
            attrs.append(f'gradientTransform="{_transform(rng)}"')
        stops = []
        if ids and rng.random() < 0.25:
            attrs.append(f'xlink:href="#{ids[rng.integers(0, len(ids))]}"')
        else:
            for _ in range(rng.integers(1, 5)):
                off = (f"{rng.uniform(0, 1):.2f}" if rng.random() < 0.7 else f"{rng.integers(0, 101)}%")
                extra = f' stop-opacity="{rng.uniform(0.2, 1):.2f}"' if rng.random() < 0.3 else ""
                if rng.random() < 0.5:
                    stops.append(f'<stop offset="{off}" stop-color="{_color(rng)}"{extra}/>')
                else:
                    stops.append(f'<stop offset="{off}" style="stop-color:{_color(rng)}"{extra}/>')
        tag = "radialGradient" if radial else "linearGradient"
        defs.append(f"<{tag} {' '.join(attrs)}>{''.join(stops)}</{tag}>")
        ids.append(gid)
    return defs, ids


def _shape(rng, side, grads):
    st = _style(rng, grads)
    xf = f' transform="{_transform(rng)}"' if rng.random() < 0.25 else ""
    k = rng.integers(0, 8)
    if k == 0:
        rx = f' rx="{_num(rng, 0, 20)}"' if rng.random() < 0.4 else ""
        ry = f' ry="{_num(rng, 0, 20)}"' if rng.random() < 0.3 else ""
        return (f'<rect x="{_num(rng, 0, side)}" y="{_num(rng, 0, side)}" width="{_num(rng, 1, side / 2)}" '
                f'height="{_num(rng, 1, side / 2)}"{rx}{ry} {st}{xf}/>')
    if k == 1:
        return f'<circle cx="{_num(rng, 0, side)}" cy="{_num(rng, 0, side)}" r="{_num(rng, 1, side / 4)}" {st}{xf}/>'
    if k == 2:
        return (f'<ellipse cx="{_num(rng, 0, side)}" cy="{_num(rng, 0, side)}" rx="{_num(rng, 1, side / 4)}" '
                f'ry="{_num(rng, 1, side / 4)}" {st}{xf}/>')
    if k == 3:
        return (f'<line x1="{_num(rng, 0, side)}" y1="{_num(rng, 0, side)}" x2="{_num(rng, 0, side)}" '
                f'y2="{_num(rng, 0, side)}" {st}{xf}/>')
    if k == 4:
        tag = "polyline" if rng.random() < 0.5 else "polygon"
        pts = " ".join(f"{_num(rng, 0, side)},{_num(rng, 0, side)}" for _ in range(rng.integers(2, 8)))
        return f'<{tag} points="{pts}" {st}{xf}/>'
    return f'<path d="{_path_data(rng, side)}" {st}{xf}/>'


def random_document(seed: int, n_shapes: int = 24) -> str:
    """A seeded SVG document using the forms the parser handles."""
    rng = np.random.default_rng(seed)
    side = int(rng.integers(64, 400))
    head = []
    k = rng.integers(0, 5)
    if k == 0:
        head.append(f'width="{side}" height="{side}"')
    elif k == 1:
        head.append(f'width="{side}px" height="{int(side * 0.8)}" viewBox="0 0 {side // 2} {side // 2}"')
    elif k == 2:
        head.append(f'width="{side // 2}pt" height="{side // 3}pt" viewBox="-10,-10 {side} {side * 0.7:.1f}" '
                    f'preserveAspectRatio="{["xMidYMid meet", "xMinYMax slice", "none", "xMaxYMin"][rng.integers(0, 4)]}"')
    elif k == 3:
        head.append(f'viewBox="0 0 {side} {side}"')
    defs, grads = _gradients(rng)
    body = []
    depth = 0
    for _ in range(n_shapes):
        r = rng.random()
        if r < 0.1:
            attrs = f' transform="{_transform(rng)}"' if rng.random() < 0.8 else ""
            if rng.random() < 0.5:
                attrs += f' fill="{_color(rng)}"'
            if rng.random() < 0.3:
                attrs += f' stroke="{_color(rng)}" stroke-width="{_num(rng, 0.5, 3)}"'
            body.append(f"<g{attrs}>")
            depth += 1
        elif r < 0.15 and depth:
            body.append("</g>")
            depth -= 1
        body.append(_shape(rng, side, grads))
    body += ["</g>"] * depth
    defs_block = f"<defs>{''.join(defs)}</defs>" if defs and rng.random() < 0.7 else "".join(defs)
    return (f'<svg xmlns="http://www.w3.org/2000/svg" xmlns:xlink="http://www.w3.org/1999/xlink" {" ".join(head)}>'
            f"\n{defs_block}\n" + "\n".join(body) + "\n</svg>")
