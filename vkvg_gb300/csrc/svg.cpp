/*
 * SVG ingestion: vkvg's include/vkvg-svg.h entry points (in vkvg, an adapter
 * over the nanoSVG parser it vendors, src/nsvg/vkvg_nsvg.c:28-136).
 *
 * The document reader here is this library's own, written from the SVG 1.1
 * specification: XML tags and attributes (comments, processing
 * instructions, declarations and CDATA sections skipped; the predefined
 * entities and character references decoded), presentation attributes and
 * the style attribute (SVG 1.1 section 6.4), lengths and units (7.10), the
 * transform attribute (7.6), viewBox and preserveAspectRatio (7.7, 7.8),
 * path data and its grammar (8.3), the basic shapes (9.2-9.7), colours
 * (4.2), gradient stops (13.2), and the elliptical-arc conversion of the
 * implementation notes (F.6.5 endpoint to centre, F.6.6 radius correction).
 * It produces the model vkvg's SVG walk reads (src/nsvg/vkvg_nsvg.c:82-136):
 * per shape an id, an opacity, a stroke width, a fill and a stroke paint
 * (none, a colour, or a gradient of which the walk uses the first stop's
 * colour) and subpaths as cubic Bezier point lists (a start point and three
 * points per segment; lines and quadratics are exact cubics), closed or not.
 *
 * Where the parser vkvg links departs from the specification in a way that
 * walk shows, this reader does what vkvg does, so that a document draws as it
 * draws in vkvg:
 *  - every drawing property, opacity and id included, is copied from the
 *    enclosing group and replaced by the element's own (group opacity is not
 *    a separate compositing step); a group's end tag inside defs still ends
 *    the enclosing group;
 *  - preserveAspectRatio defaults to none (non-uniform scaling), and the
 *    alignment defaults to xMin / yMin;
 *  - a paint url(#id) is resolved when the shape is read: a gradient
 *    defined later leaves the paint none; stops sort by offset (ties keep
 *    document order), a stop belongs to the last gradient opened, and a
 *    gradient without stops takes those of the one its xlink:href names;
 *  - colour names other than the ten vkvg's build knows (black, white,
 *    red, green, blue, yellow, cyan, magenta, grey, gray) read as grey; an
 *    alpha byte is the opacity times 255, truncated;
 *  - S and T reflect the last control point of whichever curve came before;
 *  - an arc becomes int(|sweep| / 90 deg + 1) cubics, the last ending where
 *    the ellipse's parametrisation puts it; an arc whose ends meet or whose
 *    radius is below 1e-6 becomes a line;
 *  - a closed subpath gets a line back to its start; a subpath without a
 *    segment is dropped; a shape's subpaths come last-first;
 *  - stroke widths scale by the mean of the transform's two column norms
 *    and by the mean of the viewBox scales; em is the font-size (0 unless
 *    set), ex 0.52 em; percentages refer to the viewBox read so far;
 *  - display="none" is recorded but the walk draws the shape anyway;
 *    elements this reader does not know pass their children through
 *    (a rect inside a clipPath is drawn, as in vkvg).
 * Numbers are converted exactly to double (the digits as an integer, scaled
 * by an exact power of ten where one exists) and rounded once to float.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "vkvg.h"
#include "vkvg-svg.h"
#include "vkvg_gb300.h"

namespace {

const float kPi       = 3.14159265358979323846f;
/* handle length, over the radius, of the cubic closest to a quarter circle:
   4/3 (sqrt(2) - 1) */
const float kQuarterHandle = 0.5522847498f;

enum PaintKind : uint32_t { PAINT_NONE = 0, PAINT_COLOR = 1, PAINT_LINEAR = 2, PAINT_RADIAL = 3 };

inline bool is_wsp(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v'; }
inline bool is_digit(char c) { return c >= '0' && c <= '9'; }
inline bool is_alpha(char c) { return (c >= 'a' && c <= 'z') || (c >= 'A' && c <= 'Z'); }

struct Cursor {
    const char *p, *e;
    bool        done() const { return p >= e; }
    char        peek() const { return p < e ? *p : '\0'; }
    void        skip_wsp() {
        while (p < e && is_wsp(*p))
            p++;
    }
    void skip_comma_wsp() {
        while (p < e && (is_wsp(*p) || *p == ','))
            p++;
    }
};

/* ------------------------------------------------------------- numbers */

/* m x 10^k as the double nearest to it: exact operands give a correctly
   rounded product or quotient; otherwise long double arithmetic */
double scale10(uint64_t m, int k) {
    static const double p10[] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                 1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    if (m == 0)
        return 0.0;
    if (m < (1ull << 53) && k >= -22 && k <= 22)
        return k >= 0 ? (double)m * p10[k] : (double)m / p10[-k];
    return (double)((long double)m * powl(10.0L, (long double)k));
}

/* a number of the SVG grammar: [+-] (digits [. digits*] | . digits)
   [(e|E) [+-] digits]; the exponent is taken only when digits follow it
   (so "2em" is 2 followed by a unit).  False, with c unmoved, if none. */
bool read_number(Cursor &c, double &v) {
    const char *q   = c.p;
    bool        neg = false;
    if (q < c.e && (*q == '+' || *q == '-'))
        neg = *q++ == '-';
    uint64_t m  = 0;
    int      k  = 0, nd = 0;
    auto     dg = [&](char ch, bool frac) {
        if (m < 100000000000000000ull) {
            m = m * 10 + (uint64_t)(ch - '0');
            k -= frac ? 1 : 0;
        } else if (!frac) {
            k++;
        }
    };
    while (q < c.e && is_digit(*q))
        dg(*q++, false), nd++;
    if (q < c.e && *q == '.') {
        const char *t  = q + 1;
        int         nf = 0;
        while (t < c.e && is_digit(*t))
            dg(*t++, true), nf++;
        if (nd + nf > 0)
            q = t, nd += nf;
    }
    if (nd == 0)
        return false;
    if (q < c.e && (*q == 'e' || *q == 'E')) {
        const char *t  = q + 1;
        bool        en = false;
        if (t < c.e && (*t == '+' || *t == '-'))
            en = *t++ == '-';
        if (t < c.e && is_digit(*t)) {
            int x = 0;
            while (t < c.e && is_digit(*t)) {
                if (x < 100000)
                    x = x * 10 + (*t - '0');
                t++;
            }
            k += en ? -x : x;
            q = t;
        }
    }
    v   = scale10(m, k);
    v   = neg ? -v : v;
    c.p = q;
    return true;
}

/* as read_number, rounded to float; a value beyond float's range is not a
   number this reader accepts */
bool read_float(Cursor &c, float &f) {
    const char *p0 = c.p;
    double      v;
    if (!read_number(c, v))
        return false;
    f = (float)v;
    if (!std::isfinite(f)) {
        c.p = p0;
        return false;
    }
    return true;
}

/* the number at the start of a value (0 if there is none) */
float leading_float(const std::string &s) {
    Cursor c{s.data(), s.data() + s.size()};
    c.skip_wsp();
    float f = 0.f;
    read_float(c, f);
    return f;
}

/* ------------------------------------------------------------ geometry */

/* x' = a x + c y + e, y' = b x + d y + f (SVG's matrix(a b c d e f)) */
struct Affine {
    float a = 1.f, b = 0.f, c = 0.f, d = 1.f, e = 0.f, f = 0.f;
};
/* outer after inner */
Affine compose(const Affine &outer, const Affine &inner) {
    Affine r;
    r.a = inner.a * outer.a + inner.b * outer.c;
    r.b = inner.a * outer.b + inner.b * outer.d;
    r.c = inner.c * outer.a + inner.d * outer.c;
    r.d = inner.c * outer.b + inner.d * outer.d;
    r.e = inner.e * outer.a + inner.f * outer.c + outer.e;
    r.f = inner.e * outer.b + inner.f * outer.d + outer.f;
    return r;
}
void apply(const Affine &m, float x, float y, float &ox, float &oy) {
    ox = x * m.a + y * m.c + m.e;
    oy = x * m.b + y * m.d + m.f;
}
Affine translation(float x, float y) {
    Affine m;
    m.e = x, m.f = y;
    return m;
}

/* the transform attribute: a list of functions, the last applied first */
Affine read_transform(const std::string &s) {
    Affine acc;
    Cursor c{s.data(), s.data() + s.size()};
    for (;;) {
        c.skip_comma_wsp();
        if (c.done())
            break;
        const char *n0 = c.p;
        while (!c.done() && is_alpha(c.peek()))
            c.p++;
        std::string name(n0, c.p);
        c.skip_wsp();
        if (name.empty() || c.peek() != '(') {
            c.p++; /* not a function: step over the character */
            continue;
        }
        c.p++;
        float a[6];
        int   n = 0;
        for (;;) {
            c.skip_comma_wsp();
            if (c.done() || c.peek() == ')')
                break;
            float v;
            if (!read_float(c, v)) {
                c.p++;
                continue;
            }
            if (n < 6)
                a[n] = v;
            n++;
        }
        if (!c.done())
            c.p++; /* ')' */
        Affine fn;
        bool   ok = true;
        if (name == "matrix" && n == 6) {
            fn.a = a[0], fn.b = a[1], fn.c = a[2], fn.d = a[3], fn.e = a[4], fn.f = a[5];
        } else if (name == "translate" && (n == 1 || n == 2)) {
            fn = translation(a[0], n == 2 ? a[1] : 0.f);
        } else if (name == "scale" && (n == 1 || n == 2)) {
            fn.a = a[0], fn.d = n == 2 ? a[1] : a[0];
        } else if (name == "rotate" && (n == 1 || n == 3)) {
            const float t = a[0] / 180.f * kPi, cs = cosf(t), sn = sinf(t);
            fn.a = cs, fn.b = sn, fn.c = -sn, fn.d = cs;
            if (n == 3) /* about (cx, cy): there, rotate, back */
                fn = compose(translation(a[1], a[2]), compose(fn, translation(-a[1], -a[2])));
        } else if (name == "skewX" && n == 1) {
            fn.c = tanf(a[0] / 180.f * kPi);
        } else if (name == "skewY" && n == 1) {
            fn.b = tanf(a[0] / 180.f * kPi);
        } else {
            ok = false;
        }
        if (ok)
            acc = compose(acc, fn);
    }
    return acc;
}

/* tight box of a cubic (its ends, and the extrema of each coordinate
   inside the curve, where the derivative's quadratic has a root) */
void cubic_box(const float *p, float box[4]) {
    box[0] = fminf(p[0], p[6]), box[1] = fminf(p[1], p[7]);
    box[2] = fmaxf(p[0], p[6]), box[3] = fmaxf(p[1], p[7]);
    for (int ax = 0; ax < 2; ax++) {
        const double p0 = p[ax], p1 = p[2 + ax], p2 = p[4 + ax], p3 = p[6 + ax];
        /* B'(t) / 3 = A t^2 + B t + C */
        const double A = -p0 + 3 * p1 - 3 * p2 + p3, B = 2 * (p0 - 2 * p1 + p2), C = p1 - p0;
        double       r[2];
        int          nr = 0;
        if (fabs(A) < 1e-12) {
            if (fabs(B) > 1e-12)
                r[nr++] = -C / B;
        } else {
            const double disc = B * B - 4 * A * C;
            if (disc > 1e-12) {
                const double sq = sqrt(disc);
                r[nr++]         = (-B + sq) / (2 * A);
                r[nr++]         = (-B - sq) / (2 * A);
            }
        }
        for (int i = 0; i < nr; i++) {
            const double t = r[i];
            if (!(t > 1e-12 && t < 1 - 1e-12))
                continue;
            const double u = 1 - t;
            const float  v = (float)(u * u * u * p0 + 3 * u * u * t * p1 + 3 * u * t * t * p2 + t * t * t * p3);
            box[ax]        = fminf(box[ax], v);
            box[2 + ax]    = fmaxf(box[2 + ax], v);
        }
    }
}

/* ------------------------------------------------------------ the model */

struct Subpath {
    std::vector<float> xy; /* 1 + 3n points */
    bool               closed = false;
    float              box[4] = {0, 0, 0, 0};
};

struct Paint {
    uint32_t kind = PAINT_NONE;
    uint32_t abgr = 0; /* r | g << 8 | b << 16 | a << 24 */
};

struct Shape {
    std::string          id;
    float                opacity = 1.f, stroke_width = 1.f;
    Paint                fill, stroke;
    bool                 visible = true;
    std::vector<Subpath> subpaths; /* last-first */
    float                box[4] = {0, 0, 0, 0};
};

} /* namespace */

struct _vkvg_svg_t {
    float              width = 0.f, height = 0.f;
    std::vector<Shape> shapes;
};

namespace {

/* ------------------------------------------------------------- colours */

uint32_t rgb_word(uint32_t r, uint32_t g, uint32_t b) { return r | g << 8 | b << 16; }

uint32_t read_color(const std::string &v) {
    size_t i = 0;
    while (i < v.size() && v[i] == ' ')
        i++;
    const std::string s = v.substr(i);
    if (!s.empty() && s[0] == '#') {
        size_t n = 1;
        while (n < s.size() && !is_wsp(s[n]))
            n++;
        const std::string hex = s.substr(1, n - 1);
        auto              hv  = [](char ch) -> int {
            return ch >= '0' && ch <= '9' ? ch - '0' : ch >= 'a' && ch <= 'f' ? ch - 'a' + 10
                                                  : ch >= 'A' && ch <= 'F'   ? ch - 'A' + 10
                                                                             : -1;
        };
        int d[6], nh = 0;
        for (char ch : hex) {
            if (nh == 6 || hv(ch) < 0)
                break;
            d[nh++] = hv(ch);
        }
        if (hex.size() == 6 && nh == 6)
            return rgb_word((uint32_t)(d[0] * 16 + d[1]), (uint32_t)(d[2] * 16 + d[3]), (uint32_t)(d[4] * 16 + d[5]));
        if (hex.size() == 3 && nh == 3)
            return rgb_word((uint32_t)(d[0] * 17), (uint32_t)(d[1] * 17), (uint32_t)(d[2] * 17));
        return 0; /* malformed: black, as in vkvg */
    }
    if (s.compare(0, 4, "rgb(") == 0) {
        Cursor   c{s.data() + 4, s.data() + s.size()};
        int      comp[3] = {0, 0, 0};
        bool     pct     = false;
        for (int k = 0; k < 3; k++) {
            c.skip_wsp();
            double x = 0;
            if (!read_number(c, x))
                break;
            comp[k] = (int)std::max(-1e6, std::min(1e6, x));
            if (c.peek() == '%') {
                pct = pct || k == 0;
                c.p++;
            }
            c.skip_comma_wsp();
        }
        uint32_t ch[3];
        for (int k = 0; k < 3; k++) {
            int x = pct ? comp[k] * 255 / 100 : comp[k];
            ch[k] = (uint32_t)(x < 0 ? 0 : x > 255 ? 255 : x);
        }
        return rgb_word(ch[0], ch[1], ch[2]);
    }
    static const struct {
        const char *name;
        uint32_t    rgb;
    } known[] = {{"red", 0x0000ff},   {"green", 0x008000},  {"blue", 0xff0000},    {"yellow", 0x00ffff},
                 {"cyan", 0xffff00},  {"magenta", 0xff00ff}, {"black", 0x000000},  {"grey", 0x808080},
                 {"gray", 0x808080},  {"white", 0xffffff}};
    for (const auto &k : known)
        if (s == k.name)
            return k.rgb;
    return 0x808080;
}

float read_unit_interval(const std::string &s) {
    const float f = leading_float(s);
    return f < 0.f ? 0.f : f > 1.f ? 1.f : f;
}

/* -------------------------------------------------------------- lengths */

enum Unit { U_USER, U_PX, U_PT, U_PC, U_MM, U_CM, U_IN, U_PCT, U_EM, U_EX };

struct Length {
    float v = 0.f;
    Unit  u = U_USER;
};

Length read_length(const std::string &s) {
    Length L;
    Cursor c{s.data(), s.data() + s.size()};
    c.skip_wsp();
    if (!read_float(c, L.v))
        L.v = 0.f;
    const char a = c.peek(), b = c.p + 1 < c.e ? c.p[1] : '\0';
    if (a == '%')
        L.u = U_PCT;
    else if (a == 'p' && b == 'x')
        L.u = U_PX;
    else if (a == 'p' && b == 't')
        L.u = U_PT;
    else if (a == 'p' && b == 'c')
        L.u = U_PC;
    else if (a == 'm' && b == 'm')
        L.u = U_MM;
    else if (a == 'c' && b == 'm')
        L.u = U_CM;
    else if (a == 'i' && b == 'n')
        L.u = U_IN;
    else if (a == 'e' && b == 'm')
        L.u = U_EM;
    else if (a == 'e' && b == 'x')
        L.u = U_EX;
    return L;
}

/* ---------------------------------------------------------------- style */

struct PaintSpec {
    uint32_t    kind = PAINT_COLOR; /* PAINT_NONE, PAINT_COLOR, or 9: a url */
    uint32_t    rgb  = 0;
    std::string ref;
};
const uint32_t PAINT_URL = 9;

struct Style {
    Affine      ctm;
    std::string id;
    PaintSpec   fill, stroke;
    float       opacity = 1.f, fill_opacity = 1.f, stroke_opacity = 1.f, stroke_width = 1.f, font_size = 0.f;
    bool        visible = true;
    Style() { stroke.kind = PAINT_NONE; }
};

struct GradientDef {
    std::string                             id, href;
    uint32_t                                kind = PAINT_LINEAR;
    std::vector<std::pair<float, uint32_t>> stops; /* offset, abgr; sorted */
};

struct TagAttr {
    std::string name, value;
};

/* the subpaths of one element, in its own coordinates */
struct Outline {
    std::vector<float>   pts;
    std::vector<Subpath> done;

    void point(float x, float y) { pts.push_back(x), pts.push_back(y); }
    bool empty() const { return pts.empty(); }
    void move_to(float x, float y) {
        if (pts.empty())
            point(x, y);
        else /* a moveto right after another replaces it */
            pts[pts.size() - 2] = x, pts[pts.size() - 1] = y;
    }
    void line_to(float x, float y) {
        if (pts.empty())
            return;
        const float x0 = pts[pts.size() - 2], y0 = pts[pts.size() - 1], dx = x - x0, dy = y - y0;
        point(x0 + dx / 3.f, y0 + dy / 3.f);
        point(x - dx / 3.f, y - dy / 3.f);
        point(x, y);
    }
    void cubic_to(float x1, float y1, float x2, float y2, float x, float y) {
        if (pts.empty())
            return;
        point(x1, y1), point(x2, y2), point(x, y);
    }
    /* ends the current subpath (kept if it has a segment) */
    void commit(bool closed, const Affine &m) {
        if (pts.size() >= 8) {
            if (closed)
                line_to(pts[0], pts[1]);
            Subpath sp;
            sp.closed = closed;
            sp.xy.resize(pts.size());
            for (size_t i = 0; i < pts.size(); i += 2)
                apply(m, pts[i], pts[i + 1], sp.xy[i], sp.xy[i + 1]);
            for (size_t i = 0; i + 7 < sp.xy.size(); i += 6) {
                float b[4];
                cubic_box(&sp.xy[i], b);
                if (i == 0) {
                    memcpy(sp.box, b, sizeof b);
                } else {
                    sp.box[0] = fminf(sp.box[0], b[0]), sp.box[1] = fminf(sp.box[1], b[1]);
                    sp.box[2] = fmaxf(sp.box[2], b[2]), sp.box[3] = fmaxf(sp.box[3], b[3]);
                }
            }
            done.push_back(std::move(sp));
        }
        pts.clear();
    }
};

/* ------------------------------------------------------------ path data */

/* arguments per command (0: not a command this reader draws) */
int arity(char cmd) {
    switch (cmd) {
    case 'M': case 'm': case 'L': case 'l': case 'T': case 't': return 2;
    case 'H': case 'h': case 'V': case 'v': return 1;
    case 'S': case 's': case 'Q': case 'q': return 4;
    case 'C': case 'c': return 6;
    case 'A': case 'a': return 7;
    default: return 0;
    }
}

/* the angle from u to v (F.6.5.4): the arc cosine of their normalised dot
   product, signed by their cross product */
float vec_angle(float ux, float uy, float vx, float vy) {
    float r = (ux * vx + uy * vy) / (sqrtf(ux * ux + uy * uy) * sqrtf(vx * vx + vy * vy));
    r       = r < -1.f ? -1.f : r > 1.f ? 1.f : r;
    const float a = acosf(r);
    return ux * vy - uy * vx < 0.f ? -a : a;
}

/* Elliptical arc from (x1, y1) to (x2, y2) as cubics.  The conversion is
   F.6.5 with F.6.6's radius correction, evaluated in float in the order the
   equations are written (degrees to radians as deg / 180 x pi): the number
   of pieces depends on the sweep to the last bit (a half turn sits on the
   boundary between two and three pieces), and this is the arithmetic
   vkvg's parser evaluates.  The pieces are evaluated at their ends, the
   last one included (not snapped to (x2, y2)). */
void arc_to(Outline &o, float x1, float y1, float rx, float ry, float rot_deg, bool large, bool sweep, float x2,
            float y2) {
    rx = fabsf(rx), ry = fabsf(ry);
    const float dx = x1 - x2, dy = y1 - y2;
    if (sqrtf(dx * dx + dy * dy) < 1e-6f || rx < 1e-6f || ry < 1e-6f) {
        o.line_to(x2, y2);
        return;
    }
    const float phi = rot_deg / 180.f * kPi, sp = sinf(phi), cp = cosf(phi);
    /* F.6.5.1: the half chord in the ellipse's frame */
    const float xp = cp * dx / 2.f + sp * dy / 2.f;
    const float yp = -sp * dx / 2.f + cp * dy / 2.f;
    /* F.6.6: radii too small to reach the ends grow by sqrt(lambda) */
    const float lam = (xp * xp) / (rx * rx) + (yp * yp) / (ry * ry);
    if (lam > 1.f) {
        const float g = sqrtf(lam);
        rx *= g, ry *= g;
    }
    /* F.6.5.2: the centre in that frame */
    const float rx2 = rx * rx, ry2 = ry * ry, xp2 = xp * xp, yp2 = yp * yp;
    const float num = rx2 * ry2 - rx2 * yp2 - ry2 * xp2, den = rx2 * yp2 + ry2 * xp2;
    float       k   = den > 0.f ? sqrtf(fmaxf(num, 0.f) / den) : 0.f;
    if (large == sweep)
        k = -k;
    const float cxp = k * rx * yp / ry, cyp = k * -ry * xp / rx;
    /* F.6.5.3: the centre */
    const float cx = cp * cxp - sp * cyp + (x1 + x2) / 2.f, cy = sp * cxp + cp * cyp + (y1 + y2) / 2.f;
    /* F.6.5.5-6: start angle and sweep */
    const float ux = (xp - cxp) / rx, uy = (yp - cyp) / ry, vx = (-xp - cxp) / rx, vy = (-yp - cyp) / ry;
    const float th0 = vec_angle(1.f, 0.f, ux, uy);
    float       dth = vec_angle(ux, uy, vx, vy);
    if (!sweep && dth > 0.f)
        dth -= 2.f * kPi;
    else if (sweep && dth < 0.f)
        dth += 2.f * kPi;
    if (!std::isfinite(cx) || !std::isfinite(cy) || !std::isfinite(th0) || !std::isfinite(dth)) {
        o.line_to(x2, y2); /* radii beyond float's range */
        return;
    }
    /* pieces of at most a quarter turn, each the cubic whose handles are
       4/3 tan(piece / 4) of the radius along the tangents */
    const int   n = (int)(fabsf(dth) / (0.5f * kPi) + 1.f);
    const float h = 4.f / 3.f * tanf(dth / (float)n * 0.25f);
    float       px = 0.f, py = 0.f, tx = 0.f, ty = 0.f;
    for (int i = 0; i <= n; i++) {
        const float a = th0 + dth * ((float)i / (float)n), ca = cosf(a), sa = sinf(a);
        /* the point and the handle, rotated into place */
        const float ex = ca * rx, ey = sa * ry, hx = -sa * rx * h, hy = ca * ry * h;
        const float x = ex * cp + ey * -sp + cx, y = ex * sp + ey * cp + cy;
        const float qx = hx * cp + hy * -sp, qy = hx * sp + hy * cp;
        if (i > 0)
            o.cubic_to(px + tx, py + ty, x - qx, y - qy, x, y);
        px = x, py = y, tx = qx, ty = qy;
    }
}

/* the d attribute (SVG 1.1 8.3.9), drawn into o; m: the element's
   transform, applied to each subpath as it ends */
void read_path_data(const std::string &d, Outline &o, const Affine &m) {
    Cursor c{d.data(), d.data() + d.size()};
    char   cmd = 0;
    float  cx = 0.f, cy = 0.f; /* current point */
    float  kx = 0.f, ky = 0.f; /* last control point */
    for (;;) {
        c.skip_comma_wsp();
        if (c.done())
            break;
        const char ch = c.peek();
        if (!(is_digit(ch) || ch == '.' || ch == '-' || ch == '+')) {
            cmd = ch;
            c.p++;
            if (cmd == 'M' || cmd == 'm') {
                o.commit(false, m);
            } else if (cmd == 'Z' || cmd == 'z') {
                if (!o.empty()) {
                    cx = o.pts[0], cy = o.pts[1];
                    kx = cx, ky = cy;
                    o.commit(true, m);
                }
                o.pts.clear();
                o.move_to(cx, cy); /* the next segment starts at the start */
            }
            continue;
        }
        const int n = arity(cmd);
        if (n == 0) { /* numbers after Z or after an unknown letter: skipped */
            double skip;
            if (!read_number(c, skip))
                c.p++;
            continue;
        }
        float a[7];
        int   got = 0;
        for (; got < n; got++) {
            c.skip_comma_wsp();
            if ((cmd == 'A' || cmd == 'a') && (got == 3 || got == 4) && (c.peek() == '0' || c.peek() == '1')) {
                a[got] = (float)(*c.p++ - '0'); /* a flag is one character */
                continue;
            }
            if (!read_float(c, a[got]))
                break;
        }
        if (got < n) /* a malformed argument list ends the data */
            break;
        const bool  rel = cmd >= 'a';
        const float ox = rel ? cx : 0.f, oy = rel ? cy : 0.f;
        switch (cmd) {
        case 'M': case 'm':
            cx = ox + a[0], cy = oy + a[1];
            o.move_to(cx, cy);
            kx = cx, ky = cy;
            cmd = rel ? 'l' : 'L'; /* further pairs are lines */
            break;
        case 'L': case 'l':
            cx = ox + a[0], cy = oy + a[1];
            o.line_to(cx, cy);
            kx = cx, ky = cy;
            break;
        case 'H': case 'h':
            cx = ox + a[0];
            o.line_to(cx, cy);
            kx = cx, ky = cy;
            break;
        case 'V': case 'v':
            cy = oy + a[0];
            o.line_to(cx, cy);
            kx = cx, ky = cy;
            break;
        case 'C': case 'c':
            o.cubic_to(ox + a[0], oy + a[1], ox + a[2], oy + a[3], ox + a[4], oy + a[5]);
            kx = ox + a[2], ky = oy + a[3];
            cx = ox + a[4], cy = oy + a[5];
            break;
        case 'S': case 's': {
            const float x1 = 2.f * cx - kx, y1 = 2.f * cy - ky;
            o.cubic_to(x1, y1, ox + a[0], oy + a[1], ox + a[2], oy + a[3]);
            kx = ox + a[0], ky = oy + a[1];
            cx = ox + a[2], cy = oy + a[3];
            break;
        }
        case 'Q': case 'q': case 'T': case 't': {
            float qx, qy, ex, ey;
            if (cmd == 'Q' || cmd == 'q')
                qx = ox + a[0], qy = oy + a[1], ex = ox + a[2], ey = oy + a[3];
            else
                qx = 2.f * cx - kx, qy = 2.f * cy - ky, ex = ox + a[0], ey = oy + a[1];
            /* the quadratic's exact cubic: control points 2/3 of the way to q */
            const float t = 2.f / 3.f;
            o.cubic_to(cx + t * (qx - cx), cy + t * (qy - cy), ex + t * (qx - ex), ey + t * (qy - ey), ex, ey);
            kx = qx, ky = qy;
            cx = ex, cy = ey;
            break;
        }
        case 'A': case 'a': {
            const float ex = ox + a[5], ey = oy + a[6];
            arc_to(o, cx, cy, a[0], a[1], a[2], fabsf(a[3]) > 1e-6f, fabsf(a[4]) > 1e-6f, ex, ey);
            cx = ex, cy = ey;
            kx = cx, ky = cy;
            break;
        }
        default:
            break;
        }
    }
    o.commit(false, m);
}

/* ------------------------------------------------------------ XML scan */

void append_utf8(std::string &out, uint32_t cp) {
    if (cp < 0x80) {
        out += (char)cp;
    } else if (cp < 0x800) {
        out += (char)(0xC0 | cp >> 6), out += (char)(0x80 | (cp & 63));
    } else if (cp < 0x10000) {
        out += (char)(0xE0 | cp >> 12), out += (char)(0x80 | (cp >> 6 & 63)), out += (char)(0x80 | (cp & 63));
    } else if (cp < 0x110000) {
        out += (char)(0xF0 | cp >> 18), out += (char)(0x80 | (cp >> 12 & 63));
        out += (char)(0x80 | (cp >> 6 & 63)), out += (char)(0x80 | (cp & 63));
    }
}

/* an attribute value with its entity and character references replaced */
std::string decode_entities(const char *p, const char *e) {
    std::string out;
    out.reserve((size_t)(e - p));
    while (p < e) {
        if (*p != '&') {
            out += *p++;
            continue;
        }
        const char *semi = p + 1;
        while (semi < e && semi - p < 12 && *semi != ';')
            semi++;
        if (semi >= e || *semi != ';') {
            out += *p++;
            continue;
        }
        const std::string ent(p + 1, semi);
        uint32_t          cp = 0;
        bool              ok = true;
        if (ent == "lt")
            cp = '<';
        else if (ent == "gt")
            cp = '>';
        else if (ent == "amp")
            cp = '&';
        else if (ent == "quot")
            cp = '"';
        else if (ent == "apos")
            cp = '\'';
        else if (ent.size() > 1 && ent[0] == '#') {
            const bool hex = ent[1] == 'x' || ent[1] == 'X';
            cp             = (uint32_t)strtoul(ent.c_str() + (hex ? 2 : 1), nullptr, hex ? 16 : 10);
        } else
            ok = false;
        if (!ok) {
            out += *p++;
            continue;
        }
        append_utf8(out, cp);
        p = semi + 1;
    }
    return out;
}

const char *find(const char *p, const char *e, const char *pat) {
    const size_t n = strlen(pat);
    for (; p + n <= e; p++)
        if (memcmp(p, pat, n) == 0)
            return p;
    return e;
}

struct Tag {
    bool                 end = false, self_closing = false;
    std::string          name;
    std::vector<TagAttr> attrs;
};

/* the next start or end tag at or after c; false at the end */
bool next_tag(Cursor &c, Tag &t) {
    for (;;) {
        while (!c.done() && c.peek() != '<')
            c.p++;
        if (c.done())
            return false;
        const char *s = c.p, *e = c.e;
        if (s + 4 <= e && memcmp(s, "<!--", 4) == 0) {
            const char *q = find(s + 4, e, "-->");
            c.p           = q < e ? q + 3 : e;
            continue;
        }
        if (s + 9 <= e && memcmp(s, "<![CDATA[", 9) == 0) {
            const char *q = find(s + 9, e, "]]>");
            c.p           = q < e ? q + 3 : e;
            continue;
        }
        if (s + 2 <= e && s[1] == '?') {
            const char *q = find(s + 2, e, "?>");
            c.p           = q < e ? q + 2 : e;
            continue;
        }
        if (s + 2 <= e && s[1] == '!') { /* a declaration, with its internal subset */
            int         depth = 0;
            const char *q     = s + 2;
            for (; q < e; q++) {
                if (*q == '[')
                    depth++;
                else if (*q == ']')
                    depth--;
                else if (*q == '>' && depth <= 0)
                    break;
            }
            c.p = q < e ? q + 1 : e;
            continue;
        }
        t     = Tag();
        c.p   = s + 1;
        t.end = c.peek() == '/';
        if (t.end)
            c.p++;
        c.skip_wsp();
        const char *n0 = c.p;
        while (!c.done() && !is_wsp(c.peek()) && c.peek() != '>' && c.peek() != '/')
            c.p++;
        t.name.assign(n0, c.p);
        for (;;) {
            c.skip_wsp();
            if (c.done())
                return true;
            if (c.peek() == '>') {
                c.p++;
                break;
            }
            if (c.peek() == '/') {
                c.p++;
                if (c.peek() == '>') {
                    c.p++;
                    t.self_closing = !t.end;
                    break;
                }
                continue;
            }
            const char *a0 = c.p;
            while (!c.done() && !is_wsp(c.peek()) && c.peek() != '=' && c.peek() != '>' && c.peek() != '/')
                c.p++;
            std::string name(a0, c.p);
            c.skip_wsp();
            if (c.peek() != '=') {
                if (a0 == c.p && !c.done())
                    c.p++;
                continue; /* an attribute without a value: ignored */
            }
            c.p++;
            c.skip_wsp();
            const char q = c.peek();
            if (q != '"' && q != '\'')
                continue;
            const char *v0 = ++c.p;
            while (!c.done() && c.peek() != q)
                c.p++;
            if (!t.end)
                t.attrs.push_back({name, decode_entities(v0, c.p)});
            if (!c.done())
                c.p++;
        }
        return true;
    }
}

/* -------------------------------------------------------------- reader */

const size_t kIdMax = 63; /* ids keep their first 63 bytes, as in vkvg */

struct Reader {
    _vkvg_svg_t             *doc;
    float                    dpi;
    std::vector<Style>       stack{Style()};
    std::vector<GradientDef> grads;
    bool                     in_defs = false;
    float                    vb_x = 0.f, vb_y = 0.f, vb_w = 0.f, vb_h = 0.f;
    int                      align_x = 0, align_y = 0, align_mode = 0; /* 0 min / none, 1 mid / meet, 2 max / slice */

    Style &top() { return stack.back(); }

    float diag() const { return sqrtf(vb_w * vb_w + vb_h * vb_h) / sqrtf(2.f); }
    float px(const Length &L, float origin, float extent) {
        switch (L.u) {
        case U_PT: return L.v / 72.f * dpi;
        case U_PC: return L.v / 6.f * dpi;
        case U_MM: return L.v / 25.4f * dpi;
        case U_CM: return L.v / 2.54f * dpi;
        case U_IN: return L.v * dpi;
        case U_EM: return L.v * top().font_size;
        case U_EX: return L.v * top().font_size * 0.52f;
        case U_PCT: return origin + L.v / 100.f * extent;
        default: return L.v;
        }
    }
    float px(const std::string &s, float origin, float extent) { return px(read_length(s), origin, extent); }

    PaintSpec read_paint(const std::string &v) {
        PaintSpec p;
        if (v == "none") {
            p.kind = PAINT_NONE;
        } else if (v.compare(0, 4, "url(") == 0) {
            p.kind       = PAINT_URL;
            size_t i     = 4;
            while (i < v.size() && is_wsp(v[i]))
                i++;
            if (i < v.size() && v[i] == '#')
                i++;
            size_t j = v.find(')', i);
            j        = j == std::string::npos ? v.size() : j;
            while (j > i && is_wsp(v[j - 1]))
                j--;
            p.ref = v.substr(i, std::min(j - i, kIdMax));
        } else {
            p.kind = PAINT_COLOR;
            p.rgb  = read_color(v);
        }
        return p;
    }

    void style_decls(Style &st, const std::string &s) {
        size_t i = 0;
        while (i < s.size()) {
            size_t j = s.find(';', i);
            j        = j == std::string::npos ? s.size() : j;
            const std::string decl = s.substr(i, j - i);
            const size_t      colon = decl.find(':');
            if (colon != std::string::npos) {
                size_t a = 0, b = colon;
                while (a < b && is_wsp(decl[a]))
                    a++;
                while (b > a && is_wsp(decl[b - 1]))
                    b--;
                size_t c = colon + 1, d = decl.size();
                while (c < d && is_wsp(decl[c]))
                    c++;
                while (d > c && is_wsp(decl[d - 1]))
                    d--;
                property(st, decl.substr(a, b - a), decl.substr(c, d - c));
            }
            i = j + 1;
        }
    }

    /* a presentation attribute or style property; false if not one */
    bool property(Style &st, const std::string &n, const std::string &v) {
        if (n == "style")
            style_decls(st, v);
        else if (n == "display") {
            if (v == "none")
                st.visible = false;
        } else if (n == "fill")
            st.fill = read_paint(v);
        else if (n == "stroke")
            st.stroke = read_paint(v);
        else if (n == "opacity")
            st.opacity = read_unit_interval(v);
        else if (n == "fill-opacity")
            st.fill_opacity = read_unit_interval(v);
        else if (n == "stroke-opacity")
            st.stroke_opacity = read_unit_interval(v);
        else if (n == "stroke-width")
            st.stroke_width = px(v, 0.f, diag());
        else if (n == "font-size")
            st.font_size = px(v, 0.f, diag());
        else if (n == "transform")
            st.ctm = compose(st.ctm, read_transform(v));
        else if (n == "id")
            st.id = v.substr(0, kIdMax);
        else if (n == "fill-rule" || n == "stroke-linejoin" || n == "stroke-linecap" || n == "stroke-miterlimit" ||
                 n == "stroke-dasharray" || n == "stroke-dashoffset" || n == "stop-color" || n == "stop-opacity" ||
                 n == "offset")
            ; /* read, and not used by the walk */
        else
            return false;
        return true;
    }

    const GradientDef *gradient(const std::string &id) const {
        for (size_t i = grads.size(); i-- > 0;)
            if (grads[i].id == id)
                return &grads[i];
        return nullptr;
    }

    Paint resolve(const PaintSpec &ps, float opacity) {
        Paint p;
        if (ps.kind == PAINT_COLOR) {
            p.kind = PAINT_COLOR;
            p.abgr = ps.rgb | (uint32_t)(opacity * 255.f) << 24;
        } else if (ps.kind == PAINT_URL) {
            const GradientDef *g = gradient(ps.ref);
            if (!g)
                return p;
            const GradientDef *s = g;
            for (int hop = 0; s && s->stops.empty() && hop < 64; hop++)
                s = gradient(s->href);
            if (!s || s->stops.empty())
                return p;
            p.kind = g->kind;
            p.abgr = s->stops[0].second;
        }
        return p;
    }

    void add_shape(Outline &o) {
        if (o.done.empty())
            return;
        const Style &st = top();
        Shape        sh;
        sh.id           = st.id;
        sh.opacity      = st.opacity;
        const float sx = sqrtf(st.ctm.a * st.ctm.a + st.ctm.c * st.ctm.c);
        const float sy = sqrtf(st.ctm.b * st.ctm.b + st.ctm.d * st.ctm.d);
        sh.stroke_width = st.stroke_width * ((sx + sy) * 0.5f);
        sh.fill         = resolve(st.fill, st.fill_opacity);
        sh.stroke       = resolve(st.stroke, st.stroke_opacity);
        sh.visible      = st.visible;
        sh.subpaths.assign(o.done.rbegin(), o.done.rend());
        memcpy(sh.box, sh.subpaths[0].box, sizeof sh.box);
        for (const Subpath &sp : sh.subpaths) {
            sh.box[0] = fminf(sh.box[0], sp.box[0]), sh.box[1] = fminf(sh.box[1], sp.box[1]);
            sh.box[2] = fmaxf(sh.box[2], sp.box[2]), sh.box[3] = fmaxf(sh.box[3], sp.box[3]);
        }
        doc->shapes.push_back(std::move(sh));
    }

    /* a basic shape or a path: the element's attributes in order, then its
       outline in the element's coordinates */
    void shape_element(const Tag &t) {
        stack.push_back(top());
        Style       &st = top();
        Outline      o;
        const float  W = vb_w, H = vb_h;
        std::string  d, points;
        float        x = 0.f, y = 0.f, w = 0.f, h = 0.f, rx = -1.f, ry = -1.f, r = 0.f, cx = 0.f, cy = 0.f;
        float        x1 = 0.f, y1 = 0.f, x2 = 0.f, y2 = 0.f;
        for (const TagAttr &a : t.attrs) {
            if (property(st, a.name, a.value))
                continue;
            const std::string &n = a.name, &v = a.value;
            if (n == "d")
                d = v;
            else if (n == "points")
                points = v;
            else if (n == "x")
                x = px(v, vb_x, W);
            else if (n == "y")
                y = px(v, vb_y, H);
            else if (n == "width")
                w = px(v, 0.f, W);
            else if (n == "height")
                h = px(v, 0.f, H);
            else if (n == "rx")
                rx = fabsf(px(v, 0.f, W));
            else if (n == "ry")
                ry = fabsf(px(v, 0.f, H));
            else if (n == "r")
                r = fabsf(px(v, 0.f, diag()));
            else if (n == "cx")
                cx = px(v, vb_x, W);
            else if (n == "cy")
                cy = px(v, vb_y, H);
            else if (n == "x1")
                x1 = px(v, vb_x, W);
            else if (n == "y1")
                y1 = px(v, vb_y, H);
            else if (n == "x2")
                x2 = px(v, vb_x, W);
            else if (n == "y2")
                y2 = px(v, vb_y, H);
        }
        const Affine &m = st.ctm;
        const float   K = kQuarterHandle;
        if (t.name == "path") {
            read_path_data(d, o, m);
        } else if (t.name == "rect") {
            /* rx / ry: one given stands for both; at most half the side */
            if (rx < 0.f && ry > 0.f)
                rx = ry;
            if (ry < 0.f && rx > 0.f)
                ry = rx;
            rx = fminf(fmaxf(rx, 0.f), w / 2.f);
            ry = fminf(fmaxf(ry, 0.f), h / 2.f);
            if (w != 0.f && h != 0.f) {
                if (rx < 1e-5f || ry < 1e-4f) {
                    o.move_to(x, y);
                    o.line_to(x + w, y);
                    o.line_to(x + w, y + h);
                    o.line_to(x, y + h);
                } else { /* lines between quarter-ellipse corners, from the top edge */
                    const float ax = x + rx, bx = x + w - rx, ay = y + ry, by = y + h - ry;
                    o.move_to(ax, y);
                    o.line_to(bx, y);
                    o.cubic_to(bx + rx * K, y, x + w, ay - ry * K, x + w, ay);
                    o.line_to(x + w, by);
                    o.cubic_to(x + w, by + ry * K, bx + rx * K, y + h, bx, y + h);
                    o.line_to(ax, y + h);
                    o.cubic_to(ax - rx * K, y + h, x, by + ry * K, x, by);
                    o.line_to(x, ay);
                    o.cubic_to(x, ay - ry * K, ax - rx * K, y, ax, y);
                }
                o.commit(true, m);
            }
        } else if (t.name == "circle" || t.name == "ellipse") {
            const float ex = t.name == "circle" ? r : rx, ey = t.name == "circle" ? r : ry;
            if (ex > 0.f && ey > 0.f) { /* four quarters from (cx + rx, cy), towards +y */
                o.move_to(cx + ex, cy);
                o.cubic_to(cx + ex, cy + ey * K, cx + ex * K, cy + ey, cx, cy + ey);
                o.cubic_to(cx - ex * K, cy + ey, cx - ex, cy + ey * K, cx - ex, cy);
                o.cubic_to(cx - ex, cy - ey * K, cx - ex * K, cy - ey, cx, cy - ey);
                o.cubic_to(cx + ex * K, cy - ey, cx + ex, cy - ey * K, cx + ex, cy);
                o.commit(true, m);
            }
        } else if (t.name == "line") {
            o.move_to(x1, y1);
            o.line_to(x2, y2);
            o.commit(false, m);
        } else { /* polyline, polygon */
            Cursor c{points.data(), points.data() + points.size()};
            float  pair[2];
            int    np = 0, k = 0;
            for (;;) {
                c.skip_comma_wsp();
                if (c.done() || !read_float(c, pair[k]))
                    break;
                if (++k == 2) {
                    if (np++ == 0)
                        o.move_to(pair[0], pair[1]);
                    else
                        o.line_to(pair[0], pair[1]);
                    k = 0;
                }
            }
            o.commit(t.name == "polygon", m);
        }
        add_shape(o);
        stack.pop_back();
    }

    void gradient_element(const Tag &t, uint32_t kind) {
        GradientDef g;
        g.kind = kind;
        for (const TagAttr &a : t.attrs) {
            if (a.name == "id")
                g.id = a.value.substr(0, kIdMax);
            else if (a.name == "xlink:href" || a.name == "href")
                g.href = a.value.substr(a.value.empty() ? 0 : 1, 62);
        }
        grads.push_back(std::move(g));
    }

    void stop_element(const Tag &t) {
        float    offset = 0.f, op = 1.f;
        uint32_t rgb = 0;
        auto     one = [&](const std::string &n, const std::string &v) {
            if (n == "offset")
                offset = px(v, 0.f, 1.f);
            else if (n == "stop-color")
                rgb = read_color(v);
            else if (n == "stop-opacity")
                op = read_unit_interval(v);
        };
        for (const TagAttr &a : t.attrs) {
            if (a.name != "style") {
                one(a.name, a.value);
                continue;
            }
            const std::string &s = a.value; /* the declarations of its style attribute */
            size_t             i = 0;
            while (i < s.size()) {
                size_t j = s.find(';', i);
                j        = j == std::string::npos ? s.size() : j;
                const std::string decl = s.substr(i, j - i);
                const size_t      colon = decl.find(':');
                if (colon != std::string::npos) {
                    auto trim = [](std::string v) {
                        size_t a0 = 0, b0 = v.size();
                        while (a0 < b0 && is_wsp(v[a0]))
                            a0++;
                        while (b0 > a0 && is_wsp(v[b0 - 1]))
                            b0--;
                        return v.substr(a0, b0 - a0);
                    };
                    one(trim(decl.substr(0, colon)), trim(decl.substr(colon + 1)));
                }
                i = j + 1;
            }
        }
        if (grads.empty())
            return;
        auto &stops = grads.back().stops;
        auto  at    = stops.begin();
        while (at != stops.end() && !(offset < at->first))
            ++at;
        stops.insert(at, {offset, rgb | (uint32_t)(op * 255.f) << 24});
    }

    void svg_element(const Tag &t) {
        for (const TagAttr &a : t.attrs) {
            if (property(top(), a.name, a.value))
                continue;
            if (a.name == "width") {
                doc->width = px(a.value, 0.f, 0.f);
            } else if (a.name == "height") {
                doc->height = px(a.value, 0.f, 0.f);
            } else if (a.name == "viewBox") {
                Cursor c{a.value.data(), a.value.data() + a.value.size()};
                float *dst[4] = {&vb_x, &vb_y, &vb_w, &vb_h};
                for (float *f : dst) {
                    while (!c.done() && (is_wsp(c.peek()) || c.peek() == ',' || c.peek() == '%'))
                        c.p++;
                    if (c.done() || !read_float(c, *f))
                        break;
                }
            } else if (a.name == "preserveAspectRatio") {
                const std::string &v = a.value;
                if (v.find("none") != std::string::npos) {
                    align_mode = 0;
                } else {
                    if (v.find("xMin") != std::string::npos)
                        align_x = 0;
                    else if (v.find("xMid") != std::string::npos)
                        align_x = 1;
                    else if (v.find("xMax") != std::string::npos)
                        align_x = 2;
                    if (v.find("yMin") != std::string::npos)
                        align_y = 0;
                    else if (v.find("yMid") != std::string::npos)
                        align_y = 1;
                    else if (v.find("yMax") != std::string::npos)
                        align_y = 2;
                    align_mode = v.find("slice") != std::string::npos ? 2 : 1;
                }
            }
        }
    }

    void start(const Tag &t) {
        const std::string &n = t.name;
        if (in_defs) { /* only gradients are read inside defs */
            if (n == "linearGradient")
                gradient_element(t, PAINT_LINEAR);
            else if (n == "radialGradient")
                gradient_element(t, PAINT_RADIAL);
            else if (n == "stop")
                stop_element(t);
            return;
        }
        if (n == "g") {
            stack.push_back(top());
            for (const TagAttr &a : t.attrs)
                property(top(), a.name, a.value);
        } else if (n == "path" || n == "rect" || n == "circle" || n == "ellipse" || n == "line" ||
                   n == "polyline" || n == "polygon") {
            shape_element(t);
        } else if (n == "linearGradient") {
            gradient_element(t, PAINT_LINEAR);
        } else if (n == "radialGradient") {
            gradient_element(t, PAINT_RADIAL);
        } else if (n == "stop") {
            stop_element(t);
        } else if (n == "defs") {
            in_defs = true;
        } else if (n == "svg") {
            svg_element(t);
        }
    }

    void end(const std::string &n) {
        if (n == "g") {
            if (stack.size() > 1)
                stack.pop_back();
        } else if (n == "defs") {
            in_defs = false;
        }
    }

    /* the viewBox mapping (7.8) onto the document size, with the size taken
       from the viewBox or the drawing's box where the document gives none */
    void finish() {
        float box[4] = {0, 0, 0, 0};
        for (size_t i = 0; i < doc->shapes.size(); i++) {
            const float *b = doc->shapes[i].box;
            if (i == 0) {
                memcpy(box, b, sizeof box);
            } else {
                box[0] = fminf(box[0], b[0]), box[1] = fminf(box[1], b[1]);
                box[2] = fmaxf(box[2], b[2]), box[3] = fmaxf(box[3], b[3]);
            }
        }
        if (vb_w == 0.f) {
            if (doc->width > 0.f)
                vb_w = doc->width;
            else
                vb_x = box[0], vb_w = box[2] - box[0];
        }
        if (vb_h == 0.f) {
            if (doc->height > 0.f)
                vb_h = doc->height;
            else
                vb_y = box[1], vb_h = box[3] - box[1];
        }
        if (doc->width == 0.f)
            doc->width = vb_w;
        if (doc->height == 0.f)
            doc->height = vb_h;
        float sx = vb_w > 0.f ? doc->width / vb_w : 0.f, sy = vb_h > 0.f ? doc->height / vb_h : 0.f;
        float ox = 0.f, oy = 0.f;
        if (align_mode != 0) {
            sx = sy = align_mode == 1 ? fminf(sx, sy) : fmaxf(sx, sy);
            const float fx = align_x == 0 ? 0.f : align_x == 1 ? 0.5f : 1.f;
            const float fy = align_y == 0 ? 0.f : align_y == 1 ? 0.5f : 1.f;
            ox = (doc->width - vb_w * sx) * fx;
            oy = (doc->height - vb_h * sy) * fy;
        }
        const float mean = (sx + sy) * 0.5f;
        for (Shape &sh : doc->shapes) {
            for (Subpath &sp : sh.subpaths) {
                for (size_t i = 0; i < sp.xy.size(); i += 2) {
                    sp.xy[i]     = (sp.xy[i] - vb_x) * sx + ox;
                    sp.xy[i + 1] = (sp.xy[i + 1] - vb_y) * sy + oy;
                }
                sp.box[0] = (sp.box[0] - vb_x) * sx + ox, sp.box[2] = (sp.box[2] - vb_x) * sx + ox;
                sp.box[1] = (sp.box[1] - vb_y) * sy + oy, sp.box[3] = (sp.box[3] - vb_y) * sy + oy;
            }
            sh.box[0] = (sh.box[0] - vb_x) * sx + ox, sh.box[2] = (sh.box[2] - vb_x) * sx + ox;
            sh.box[1] = (sh.box[1] - vb_y) * sy + oy, sh.box[3] = (sh.box[3] - vb_y) * sy + oy;
            sh.stroke_width *= mean;
        }
    }
};

_vkvg_svg_t *parse_text(const char *p, size_t n, float dpi) {
    _vkvg_svg_t *doc = new (std::nothrow) _vkvg_svg_t();
    if (!doc)
        return nullptr;
    try {
        Reader rd;
        rd.doc = doc;
        rd.dpi = dpi;
        Cursor c{p, p + n};
        Tag    t;
        while (next_tag(c, t)) {
            if (!t.end)
                rd.start(t);
            if (t.end || t.self_closing)
                rd.end(t.name);
        }
        rd.finish();
    } catch (const std::bad_alloc &) {
        delete doc;
        return nullptr;
    }
    return doc;
}

_vkvg_svg_t *parse_file(const char *path, float dpi) {
    if (!path)
        return nullptr;
    FILE *f = fopen(path, "rb");
    if (!f)
        return nullptr;
    std::string text;
    char        buf[65536];
    size_t      k;
    while ((k = fread(buf, 1, sizeof buf, f)) > 0)
        text.append(buf, k);
    const bool bad = ferror(f) != 0;
    fclose(f);
    return bad ? nullptr : parse_text(text.data(), text.size(), dpi);
}

/* the walk's colour: ABGR bytes over 255, alpha times the shape opacity
   (src/nsvg/vkvg_nsvg.c:30-36) */
void set_color(VkvgContext ctx, uint32_t c, float opacity) {
    const float a = (float)(c >> 24 & 255) / 255.f, b = (float)(c >> 16 & 255) / 255.f;
    const float g = (float)(c >> 8 & 255) / 255.f, r = (float)(c & 255) / 255.f;
    vkvg_set_source_rgba(ctx, r, g, b, a * opacity);
}

VkvgSurface surface_from(VkvgDevice dev, _vkvg_svg_t *svg) {
    if (!svg)
        return nullptr;
    VkvgSurface surf = vkvg_surface_create(dev, (uint32_t)svg->width, (uint32_t)svg->height);
    if (surf) {
        VkvgContext ctx = vkvg_create(surf);
        vkvg_svg_render(svg, ctx, nullptr);
        vkvg_destroy(ctx);
    }
    delete svg;
    return surf;
}

float device_dpi(VkvgDevice dev) {
    int h = 96, v = 96;
    if (dev)
        vkvg_device_get_dpy(dev, &h, &v);
    return (float)h;
}

} /* namespace */

extern "C" {

VkvgSvg vkvg_svg_load(const char *svgFilePath) { return parse_file(svgFilePath, 96.f); }

VkvgSvg vkvg_svg_load_fragment(char *svgFragment) {
    return svgFragment ? parse_text(svgFragment, strlen(svgFragment), 96.f) : nullptr;
}

void vkvg_svg_destroy(VkvgSvg svg) { delete svg; }

void vkvg_svg_get_dimensions(VkvgSvg svg, uint32_t *width, uint32_t *height) {
    if (!svg)
        return;
    if (width)
        *width = (uint32_t)svg->width;
    if (height)
        *height = (uint32_t)svg->height;
}

/* the walk of src/nsvg/vkvg_nsvg.c:82-136: inside save / restore, even-odd
   fill, black to start; per shape (or per shape whose id is id) a new path
   of its subpaths at its stroke width, filled in its fill colour and then
   stroked in its stroke colour; a paint without a colour (a radial
   gradient) keeps the current source, and a shape with neither paint is
   stroked in it */
void vkvg_svg_render(VkvgSvg svg, VkvgContext ctx, const char *id) {
    if (!svg || !ctx)
        return;
    vkvg_save(ctx);
    vkvg_set_fill_rule(ctx, VKVG_FILL_RULE_EVEN_ODD);
    vkvg_set_source_rgba(ctx, 0.f, 0.f, 0.f, 1.f);
    for (const Shape &sh : svg->shapes) {
        if (id && sh.id != id)
            continue;
        vkvg_new_path(ctx);
        vkvg_set_line_width(ctx, sh.stroke_width);
        for (const Subpath &sp : sh.subpaths) {
            const float *p = sp.xy.data();
            vkvg_move_to(ctx, p[0], p[1]);
            for (size_t i = 2; i + 5 < sp.xy.size(); i += 6)
                vkvg_curve_to(ctx, p[i], p[i + 1], p[i + 2], p[i + 3], p[i + 4], p[i + 5]);
            if (sp.closed)
                vkvg_close_path(ctx);
        }
        if (sh.fill.kind == PAINT_COLOR || sh.fill.kind == PAINT_LINEAR)
            set_color(ctx, sh.fill.abgr, sh.opacity);
        if (sh.fill.kind != PAINT_NONE) {
            if (sh.stroke.kind == PAINT_NONE) {
                vkvg_fill(ctx);
                continue;
            }
            vkvg_fill_preserve(ctx);
        }
        if (sh.stroke.kind == PAINT_COLOR || sh.stroke.kind == PAINT_LINEAR)
            set_color(ctx, sh.stroke.abgr, sh.opacity);
        vkvg_stroke(ctx);
    }
    vkvg_restore(ctx);
}

VkvgSurface vkvg_surface_create_from_svg(VkvgDevice dev, uint32_t width, uint32_t height, const char *svgFilePath) {
    (void)width, (void)height;
    return surface_from(dev, parse_file(svgFilePath, device_dpi(dev)));
}

VkvgSurface vkvg_surface_create_from_svg_fragment(VkvgDevice dev, uint32_t width, uint32_t height,
                                                  char *svgFragment) {
    (void)width, (void)height;
    if (!svgFragment)
        return nullptr;
    return surface_from(dev, parse_text(svgFragment, strlen(svgFragment), device_dpi(dev)));
}

uint32_t vkvg_gb300_svg_shape_count(VkvgSvg svg) { return svg ? (uint32_t)svg->shapes.size() : 0u; }

int vkvg_gb300_svg_shape(VkvgSvg svg, uint32_t i, char id[64], uint32_t u[6], float f[6]) {
    if (!svg || i >= svg->shapes.size())
        return -1;
    const Shape &sh = svg->shapes[i];
    if (id) {
        memset(id, 0, 64);
        memcpy(id, sh.id.data(), std::min<size_t>(sh.id.size(), 63));
    }
    if (u) {
        u[0] = sh.fill.kind, u[1] = sh.fill.abgr, u[2] = sh.stroke.kind, u[3] = sh.stroke.abgr;
        u[4] = sh.visible ? 1u : 0u, u[5] = (uint32_t)sh.subpaths.size();
    }
    if (f) {
        f[0] = sh.opacity, f[1] = sh.stroke_width;
        memcpy(f + 2, sh.box, 4 * sizeof(float));
    }
    return 0;
}

int vkvg_gb300_svg_path(VkvgSvg svg, uint32_t shape, uint32_t path, float *pts, uint32_t cap_points, uint32_t *npts,
                        uint32_t *closed) {
    if (!svg || shape >= svg->shapes.size() || path >= svg->shapes[shape].subpaths.size())
        return -1;
    const Subpath &sp = svg->shapes[shape].subpaths[path];
    const uint32_t n  = (uint32_t)(sp.xy.size() / 2);
    if (npts)
        *npts = n;
    if (closed)
        *closed = sp.closed ? 1u : 0u;
    if (pts && cap_points)
        memcpy(pts, sp.xy.data(), sizeof(float) * 2 * std::min(n, cap_points));
    return 0;
}

} /* extern "C" */
