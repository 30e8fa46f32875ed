/* SVG ingestion: vkvg's SVG entry points (src/nsvg/vkvg_nsvg.c:28-136,
 * include/vkvg-svg.h) over a parser written here.
 *
 * vkvg parses with nanoSVG (src/nsvg/nanosvg.h, vendored in its tree) and
 * walks the resulting shape list.  The parser below restates nanoSVG's
 * published behaviour for everything that walk reads: the image size, and per
 * shape its id, opacity, scaled stroke width, fill and stroke paint (colour,
 * or the first stop of a gradient) and its paths as cubic Beziers in device
 * units (lines become cubics with control points at thirds, arcs are split
 * into quarter-turn cubics, rectangles, circles and ellipses use the 90-degree
 * kappa constant, transforms and the viewBox are applied to the points).  The
 * numeric steps follow nanoSVG's order of float operations, so on the same
 * C library its points agree with nanoSVG's to the last bit; tests hold them
 * to 1e-3 px.  nanoSVG is built in vkvg without NANOSVG_ALL_COLOR_KEYWORDS, so
 * ten colour names are known and any other name is grey.  Parsed but unused
 * by the render (dashes, joins, caps, miter, fill rule, gradient geometry)
 * is not kept.
 */
#include "host.h"

#include "../../include/vkvg-svg.h"

#include <algorithm>
#include <math.h>
#include <new>
#include <stdio.h>
#include <stdlib.h>
#include <string>
#include <vector>

namespace {

enum { PAINT_NONE = 0, PAINT_COLOR = 1, PAINT_LINEAR = 2, PAINT_RADIAL = 3 };

struct SvgPath {
    std::vector<float> pts; /* x0 y0, then (c1 c2 p) per cubic */
    bool               closed = false;
    float              bounds[4];
};
struct SvgShape {
    char                 id[64];
    uint8_t              fill_type = PAINT_NONE, stroke_type = PAINT_NONE;
    uint32_t             fill_color = 0, stroke_color = 0; /* ABGR (r in the low byte); gradients: first stop */
    float                opacity = 1, stroke_width = 1;
    bool                 visible = true;
    float                bounds[4];
    std::vector<SvgPath> paths; /* in nanoSVG's list order (last parsed first) */
};

} /* namespace */

/* a parsed document (nanoSVG's NSVGimage) */
struct _vkvg_svg_t {
    float                 width = 0, height = 0;
    std::vector<SvgShape> shapes;
};

namespace {

/* ---- characters and numbers (nanoSVG's tokenizer rules).  nanoSVG's space
   test is strchr(" \t\n\v\f\r", c), which also holds for '\0', so its
   space-skipping loops run on past the terminators its in-place tokenizer
   writes, into the rest of the document buffer: a tag whose last attribute
   is followed by a space reads the next tag as its attributes, trailing
   spaces in path data or a style value continue into the following
   attributes.  The same test and the same in-place buffer reproduce that
   here; the buffer ends in a sentinel so that no scan leaves it. */
bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r' || c == '\0';
}
bool is_digit(char c) { return c >= '0' && c <= '9'; }
bool is_num(char c) { return is_digit(c) || c == '+' || c == '-' || c == '.' || c == 'e' || c == 'E'; }

/* decimal text to double: integer digits, fraction digits over 10^n, then the
   exponent as a power of ten, all in double (locale independent) */
double parse_double(const char *s) {
    double sign = 1.0, res = 0.0;
    bool   any  = false;
    if (*s == '+')
        s++;
    else if (*s == '-') {
        sign = -1.0;
        s++;
    }
    char *end = nullptr;
    if (is_digit(*s)) {
        long long ip = strtoll(s, &end, 10);
        if (end != s) {
            res = (double)ip;
            any = true;
            s   = end;
        }
    }
    if (*s == '.') {
        s++;
        if (is_digit(*s)) {
            long long fp = strtoll(s, &end, 10);
            if (end != s) {
                res += (double)fp / pow(10.0, (double)(end - s));
                any = true;
                s   = end;
            }
        }
    }
    if (!any)
        return 0.0;
    if (*s == 'e' || *s == 'E') {
        s++;
        long ex = strtol(s, &end, 10);
        if (end != s)
            res *= pow(10.0, (double)ex);
    }
    return res * sign;
}

/* copy one number token ([sign] digits [. digits] [e [sign] digits]; a lone
   leading zero ends the integer part; "em" / "ex" are units) into it */
const char *scan_number(const char *s, char *it, int size) {
    int  n    = 0;
    auto push = [&](char c) {
        if (n < size - 1)
            it[n++] = c;
    };
    if (*s == '-' || *s == '+')
        push(*s++);
    if (*s == '0') {
        push(*s++);
    } else {
        while (is_digit(*s))
            push(*s++);
    }
    if (*s == '.') {
        push(*s++);
        while (is_digit(*s))
            push(*s++);
    }
    if ((*s == 'e' || *s == 'E') && s[1] != 'm' && s[1] != 'x') {
        push(*s++);
        if (*s == '-' || *s == '+')
            push(*s++);
        while (is_digit(*s))
            push(*s++);
    }
    it[n] = '\0';
    return s;
}

/* next path-data item: a number, or a one-character command */
const char *next_item(const char *s, char *it) {
    it[0] = '\0';
    while (is_space(*s) || *s == ',')
        s++;
    if (!*s)
        return s;
    if (*s == '-' || *s == '+' || *s == '.' || is_digit(*s))
        return scan_number(s, it, 64);
    it[0] = *s++;
    it[1] = '\0';
    return s;
}
/* an arc flag: a single 0 or 1 (flags may be written without separators) */
const char *next_flag(const char *s, char *it) {
    it[0] = '\0';
    while (is_space(*s) || *s == ',')
        s++;
    if (*s == '0' || *s == '1') {
        it[0] = *s++;
        it[1] = '\0';
    }
    return s;
}

/* ---- colours: #rgb, #rrggbb, rgb(r,g,b) / rgb(r%,g%,b%), ten names */
uint32_t rgb(uint32_t r, uint32_t g, uint32_t b) { return r | (g << 8) | (b << 16); }
uint32_t parse_color(const char *str) {
    while (*str == ' ')
        str++;
    if (*str == '#') {
        const char *h = str + 1;
        int         n = 0;
        while (h[n] && !is_space(h[n]))
            n++;
        unsigned c = 0;
        if (n == 6) {
            sscanf(h, "%x", &c);
        } else if (n == 3) {
            sscanf(h, "%x", &c);
            c = (c & 0xfu) | ((c & 0xf0u) << 4) | ((c & 0xf00u) << 8);
            c |= c << 4;
        }
        return rgb((c >> 16) & 0xffu, (c >> 8) & 0xffu, c & 0xffu);
    }
    if (strncmp(str, "rgb(", 4) == 0) {
        int  r = -1, g = -1, b = -1;
        char s1[32] = "", s2[32] = "";
        sscanf(str + 4, "%d%31[%%, \t]%d%31[%%, \t]%d", &r, s1, &g, s2, &b);
        if (strchr(s1, '%'))
            return rgb((uint32_t)((r * 255) / 100), (uint32_t)((g * 255) / 100), (uint32_t)((b * 255) / 100));
        return rgb((uint32_t)r, (uint32_t)g, (uint32_t)b);
    }
    static const struct {
        const char *name;
        uint32_t    c;
    } names[] = {{"red", 0x0000ffu},    {"green", 0x008000u}, {"blue", 0xff0000u},  {"yellow", 0x00ffffu},
                 {"cyan", 0xffff00u},   {"magenta", 0xff00ffu}, {"black", 0x000000u}, {"grey", 0x808080u},
                 {"gray", 0x808080u},   {"white", 0xffffffu}};
    for (const auto &e : names)
        if (strcmp(e.name, str) == 0)
            return e.c;
    return rgb(128, 128, 128);
}
float clamp01(double v) {
    float f = (float)v;
    return f < 0.0f ? 0.0f : (f > 1.0f ? 1.0f : f);
}

/* ---- units */
enum { U_USER, U_PX, U_PT, U_PC, U_MM, U_CM, U_IN, U_PERCENT, U_EM, U_EX };
int parse_units(const char *u) {
    if (u[0] == 'p' && u[1] == 'x')
        return U_PX;
    if (u[0] == 'p' && u[1] == 't')
        return U_PT;
    if (u[0] == 'p' && u[1] == 'c')
        return U_PC;
    if (u[0] == 'm' && u[1] == 'm')
        return U_MM;
    if (u[0] == 'c' && u[1] == 'm')
        return U_CM;
    if (u[0] == 'i' && u[1] == 'n')
        return U_IN;
    if (u[0] == '%')
        return U_PERCENT;
    if (u[0] == 'e' && u[1] == 'm')
        return U_EM;
    if (u[0] == 'e' && u[1] == 'x')
        return U_EX;
    return U_USER;
}
struct Coord {
    float v;
    int   units;
};
Coord parse_coord_raw(const char *str) {
    char buf[64];
    Coord c;
    c.units = parse_units(scan_number(str, buf, 64));
    c.v     = (float)parse_double(buf);
    return c;
}

/* ---- 2x3 transforms [a b c d e f]: x' = a x + c y + e, y' = b x + d y + f */
struct Xf {
    float t[6];
};
Xf xf_identity() { return Xf{{1, 0, 0, 1, 0, 0}}; }
Xf xf_translate(float tx, float ty) { return Xf{{1, 0, 0, 1, tx, ty}}; }
Xf xf_scale(float sx, float sy) { return Xf{{sx, 0, 0, sy, 0, 0}}; }
/* t = t then s (t's map followed by s's) */
void xf_then(Xf &t, const Xf &s) {
    const float *a = t.t, *b = s.t;
    const float  t0 = a[0] * b[0] + a[1] * b[2];
    const float  t2 = a[2] * b[0] + a[3] * b[2];
    const float  t4 = a[4] * b[0] + a[5] * b[2] + b[4];
    const float  t1 = a[0] * b[1] + a[1] * b[3];
    const float  t3 = a[2] * b[1] + a[3] * b[3];
    const float  t5 = a[4] * b[1] + a[5] * b[3] + b[5];
    t               = Xf{{t0, t1, t2, t3, t4, t5}};
}
/* t = s then t */
void xf_before(Xf &t, const Xf &s) {
    Xf r = s;
    xf_then(r, t);
    t = r;
}
void xf_point(const Xf &m, float x, float y, float *ox, float *oy) {
    *ox = x * m.t[0] + y * m.t[2] + m.t[4];
    *oy = x * m.t[1] + y * m.t[3] + m.t[5];
}
void xf_vec(const Xf &m, float x, float y, float *ox, float *oy) {
    *ox = x * m.t[0] + y * m.t[2];
    *oy = x * m.t[1] + y * m.t[3];
}
float xf_avg_scale(const Xf &m) {
    const float sx = sqrtf(m.t[0] * m.t[0] + m.t[2] * m.t[2]);
    const float sy = sqrtf(m.t[1] * m.t[1] + m.t[3] * m.t[3]);
    return (sx + sy) * 0.5f;
}

constexpr float SVG_PI    = 3.14159265358979323846264338327f;
constexpr float SVG_KAPPA = 0.5522847493f; /* cubic handle length of a quarter circle */

/* arguments of one transform function: the numbers between its parentheses;
   returns the characters consumed (to the closing parenthesis) */
int transform_args(const char *str, float *args, int max_n, int *na) {
    *na             = 0;
    const char *ptr = str;
    while (*ptr && *ptr != '(')
        ptr++;
    if (!*ptr)
        return 1;
    const char *end = ptr;
    while (*end && *end != ')')
        end++;
    if (!*end)
        return 1;
    char it[64];
    while (ptr < end) {
        if (*ptr == '-' || *ptr == '+' || *ptr == '.' || is_digit(*ptr)) {
            if (*na >= max_n)
                return 0;
            ptr           = scan_number(ptr, it, 64);
            args[(*na)++] = (float)parse_double(it);
        } else {
            ptr++;
        }
    }
    return (int)(end - str);
}
/* a transform list, each function applied before those already read */
Xf parse_transform(const char *str) {
    Xf xf = xf_identity();
    while (*str) {
        float args[6] = {0, 0, 0, 0, 0, 0};
        int   na = 0, len;
        Xf    t;
        if (strncmp(str, "matrix", 6) == 0) {
            len = transform_args(str, args, 6, &na);
            if (na != 6) {
                /* a matrix() without six numbers is skipped (nanoSVG applies
                   whatever its scratch matrix held) */
                str += len > 0 ? len : 1;
                continue;
            }
            t = Xf{{args[0], args[1], args[2], args[3], args[4], args[5]}};
        } else if (strncmp(str, "translate", 9) == 0) {
            len = transform_args(str, args, 2, &na);
            if (na == 1)
                args[1] = 0.0f;
            t = xf_translate(args[0], args[1]);
        } else if (strncmp(str, "scale", 5) == 0) {
            len = transform_args(str, args, 2, &na);
            if (na == 1)
                args[1] = args[0];
            t = xf_scale(args[0], args[1]);
        } else if (strncmp(str, "rotate", 6) == 0) {
            len = transform_args(str, args, 3, &na);
            if (na == 1)
                args[1] = args[2] = 0.0f;
            t = xf_identity();
            if (na > 1)
                xf_then(t, xf_translate(-args[1], -args[2]));
            const float a = args[0] / 180.0f * SVG_PI, cs = cosf(a), sn = sinf(a);
            xf_then(t, Xf{{cs, sn, -sn, cs, 0, 0}});
            if (na > 1)
                xf_then(t, xf_translate(args[1], args[2]));
        } else if (strncmp(str, "skewX", 5) == 0) {
            len = transform_args(str, args, 1, &na);
            t   = Xf{{1, 0, tanf(args[0] / 180.0f * SVG_PI), 1, 0, 0}};
        } else if (strncmp(str, "skewY", 5) == 0) {
            len = transform_args(str, args, 1, &na);
            t   = Xf{{1, tanf(args[0] / 180.0f * SVG_PI), 0, 1, 0, 0}};
        } else {
            str++;
            continue;
        }
        /* too many arguments consume nothing (where nanoSVG would loop on
           the same function forever); step past it */
        str += len > 0 ? len : 1;
        xf_before(xf, t);
    }
    return xf;
}

/* ---- bounds of a cubic (x0 y0 c1 c2 p, 8 floats): end points, then the
   curve's extremes where its derivative vanishes, evaluated in double */
void cubic_bounds(float *b, const float *c) {
    b[0] = fminf(c[0], c[6]);
    b[1] = fminf(c[1], c[7]);
    b[2] = fmaxf(c[0], c[6]);
    b[3] = fmaxf(c[1], c[7]);
    auto inside = [&](const float *p) { return p[0] >= b[0] && p[0] <= b[2] && p[1] >= b[1] && p[1] <= b[3]; };
    if (inside(c + 2) && inside(c + 4))
        return;
    const double eps = 1e-12;
    for (int k = 0; k < 2; k++) {
        const double p0 = c[k], p1 = c[2 + k], p2 = c[4 + k], p3 = c[6 + k];
        const double a  = -3.0 * p0 + 9.0 * p1 - 9.0 * p2 + 3.0 * p3;
        const double bb = 6.0 * p0 - 12.0 * p1 + 6.0 * p2;
        const double cc = 3.0 * p1 - 3.0 * p0;
        double       roots[2];
        int          n = 0;
        if (fabs(a) < eps) {
            if (fabs(bb) > eps) {
                const double t = -cc / bb;
                if (t > eps && t < 1.0 - eps)
                    roots[n++] = t;
            }
        } else {
            const double disc = bb * bb - 4.0 * cc * a;
            if (disc > eps) {
                double t = (-bb + sqrt(disc)) / (2.0 * a);
                if (t > eps && t < 1.0 - eps)
                    roots[n++] = t;
                t = (-bb - sqrt(disc)) / (2.0 * a);
                if (t > eps && t < 1.0 - eps)
                    roots[n++] = t;
            }
        }
        for (int j = 0; j < n; j++) {
            const double t = roots[j], it = 1.0 - t;
            const double v = it * it * it * p0 + 3.0 * it * it * t * p1 + 3.0 * it * t * t * p2 + t * t * t * p3;
            b[k]           = fminf(b[k], (float)v);
            b[2 + k]       = fmaxf(b[2 + k], (float)v);
        }
    }
}

/* the inherited style of an element (nanoSVG's attribute stack entry) */
struct Style {
    char     id[64];
    Xf       xf;
    uint32_t fill_color, stroke_color;
    float    opacity, fill_opacity, stroke_opacity, stroke_width, font_size;
    char     fill_ref[64], stroke_ref[64];
    uint32_t stop_color;
    float    stop_opacity, stop_offset;
    uint8_t  has_fill, has_stroke; /* 0 none, 1 colour, 2 url(#id) */
    bool     visible;
};
struct GradStop {
    uint32_t color;
    float    offset;
};
struct GradDef {
    char                  id[64], ref[64];
    uint8_t               type; /* PAINT_LINEAR / PAINT_RADIAL */
    std::vector<GradStop> stops;
};

constexpr int STYLE_DEPTH = 128;

struct Parser {
    Style                 st[STYLE_DEPTH];
    int                   head = 0;
    std::vector<float>    pts;   /* the subpath being built */
    std::vector<SvgPath>  plist; /* paths of the element being built, in parse order */
    std::vector<GradDef>  grads; /* in definition order; a lookup takes the latest */
    _vkvg_svg_t          *img;
    float                 view_minx = 0, view_miny = 0, view_w = 0, view_h = 0;
    int                   align_x = 0, align_y = 0, align_type = 0; /* min / mid / max; none / meet / slice */
    float                 dpi;
    bool                  in_defs = false;

    Style &cur() { return st[head]; }
    void   push() {
        if (head < STYLE_DEPTH - 1) {
            st[head + 1] = st[head];
            head++;
        }
    }
    void pop() {
        if (head > 0)
            head--;
    }
    float orig_x() const { return view_minx; }
    float orig_y() const { return view_miny; }
    float width() const { return view_w; }
    float height() const { return view_h; }
    float diag() const { return sqrtf(view_w * view_w + view_h * view_h) / sqrtf(2.0f); }

    float to_px(Coord c, float orig, float length) {
        switch (c.units) {
        case U_PT: return c.v / 72.0f * dpi;
        case U_PC: return c.v / 6.0f * dpi;
        case U_MM: return c.v / 25.4f * dpi;
        case U_CM: return c.v / 2.54f * dpi;
        case U_IN: return c.v * dpi;
        case U_EM: return c.v * cur().font_size;
        case U_EX: return c.v * cur().font_size * 0.52f;
        case U_PERCENT: return orig + c.v / 100.0f * length;
        default: return c.v;
        }
    }
    float coord(const char *s, float orig, float length) { return to_px(parse_coord_raw(s), orig, length); }

    /* ---- points of the current subpath */
    void add_point(float x, float y) {
        pts.push_back(x);
        pts.push_back(y);
    }
    void move_to(float x, float y) {
        if (!pts.empty()) {
            pts[pts.size() - 2] = x;
            pts[pts.size() - 1] = y;
        } else {
            add_point(x, y);
        }
    }
    void line_to(float x, float y) {
        if (pts.empty())
            return;
        const float px = pts[pts.size() - 2], py = pts[pts.size() - 1];
        const float dx = x - px, dy = y - py;
        add_point(px + dx / 3.0f, py + dy / 3.0f);
        add_point(x - dx / 3.0f, y - dy / 3.0f);
        add_point(x, y);
    }
    void cubic_to(float x1, float y1, float x2, float y2, float x, float y) {
        add_point(x1, y1);
        add_point(x2, y2);
        add_point(x, y);
    }
    /* close off the subpath as a path of the element, in device units */
    void add_path(bool closed) {
        if (pts.size() / 2 < 4)
            return;
        if (closed)
            line_to(pts[0], pts[1]);
        SvgPath path;
        path.closed     = closed;
        const size_t np = pts.size() / 2;
        path.pts.resize(np * 2);
        for (size_t i = 0; i < np; i++)
            xf_point(cur().xf, pts[2 * i], pts[2 * i + 1], &path.pts[2 * i], &path.pts[2 * i + 1]);
        for (size_t i = 0; i + 1 < np; i += 3) {
            float b[4];
            cubic_bounds(b, &path.pts[2 * i]);
            if (i == 0) {
                memcpy(path.bounds, b, sizeof(b));
            } else {
                path.bounds[0] = fminf(path.bounds[0], b[0]);
                path.bounds[1] = fminf(path.bounds[1], b[1]);
                path.bounds[2] = fmaxf(path.bounds[2], b[2]);
                path.bounds[3] = fmaxf(path.bounds[3], b[3]);
            }
        }
        plist.push_back(std::move(path));
    }

    bool parse_attr(const char *name, const char *value);
    void parse_style(const char *str);
    void parse_attribs(const char **attr);
    const GradDef *find_grad(const char *id) const;
    void           add_shape();
    void           parse_path(const char **attr);
    void           arc_to(float *cpx, float *cpy, const float *args, bool rel);
    void           parse_rect(const char **attr);
    void           parse_ellipse(const char **attr, bool circle);
    void           parse_line(const char **attr);
    void           parse_poly(const char **attr, bool closed);
    void           parse_svg(const char **attr);
    void           parse_gradient(const char **attr, uint8_t type);
    void           parse_stop(const char **attr);
    void           start_element(const char *el, const char **attr);
    void           end_element(const char *el);
    void           scale_to_viewbox(const char *units);
};

void copy_id(char *dst, const char *src) {
    strncpy(dst, src, 63);
    dst[63] = '\0';
}
/* url(#id) -> id (at most 63 characters) */
void parse_url(char *id, const char *str) {
    str += 4;
    if (*str == '#')
        str++;
    int i = 0;
    while (i < 63 && *str && *str != ')')
        id[i++] = *str++;
    id[i] = '\0';
}

bool Parser::parse_attr(const char *name, const char *value) {
    Style &a = cur();
    if (strcmp(name, "style") == 0) {
        parse_style(value);
    } else if (strcmp(name, "display") == 0) {
        if (strcmp(value, "none") == 0)
            a.visible = false; /* display:inline does not undo an ancestor's none */
    } else if (strcmp(name, "fill") == 0) {
        if (strcmp(value, "none") == 0) {
            a.has_fill = 0;
        } else if (strncmp(value, "url(", 4) == 0) {
            a.has_fill = 2;
            parse_url(a.fill_ref, value);
        } else {
            a.has_fill   = 1;
            a.fill_color = parse_color(value);
        }
    } else if (strcmp(name, "opacity") == 0) {
        a.opacity = clamp01(parse_double(value));
    } else if (strcmp(name, "fill-opacity") == 0) {
        a.fill_opacity = clamp01(parse_double(value));
    } else if (strcmp(name, "stroke") == 0) {
        if (strcmp(value, "none") == 0) {
            a.has_stroke = 0;
        } else if (strncmp(value, "url(", 4) == 0) {
            a.has_stroke = 2;
            parse_url(a.stroke_ref, value);
        } else {
            a.has_stroke   = 1;
            a.stroke_color = parse_color(value);
        }
    } else if (strcmp(name, "stroke-width") == 0) {
        a.stroke_width = coord(value, 0.0f, diag());
    } else if (strcmp(name, "stroke-opacity") == 0) {
        a.stroke_opacity = clamp01(parse_double(value));
    } else if (strcmp(name, "font-size") == 0) {
        a.font_size = coord(value, 0.0f, diag());
    } else if (strcmp(name, "transform") == 0) {
        xf_before(a.xf, parse_transform(value));
    } else if (strcmp(name, "stop-color") == 0) {
        a.stop_color = parse_color(value);
    } else if (strcmp(name, "stop-opacity") == 0) {
        a.stop_opacity = clamp01(parse_double(value));
    } else if (strcmp(name, "offset") == 0) {
        a.stop_offset = coord(value, 0.0f, 1.0f);
    } else if (strcmp(name, "id") == 0) {
        copy_id(a.id, value);
    } else if (strcmp(name, "stroke-dasharray") == 0 || strcmp(name, "stroke-dashoffset") == 0 ||
               strcmp(name, "stroke-linecap") == 0 || strcmp(name, "stroke-linejoin") == 0 ||
               strcmp(name, "stroke-miterlimit") == 0 || strcmp(name, "fill-rule") == 0) {
        /* recognised; the render does not use them */
    } else {
        return false;
    }
    return true;
}
/* "name: value; ..." with both sides trimmed, each at most 511 characters */
void Parser::parse_style(const char *str) {
    while (*str) {
        while (is_space(*str))
            str++;
        const char *start = str;
        while (*str && *str != ';')
            str++;
        const char *end = str;
        while (end > start && (*end == ';' || is_space(*end)))
            end--;
        end++;
        const char *sep = start;
        while (sep < end && *sep != ':')
            sep++;
        const char *nend = sep;
        while (nend > start && (*nend == ':' || is_space(*nend)))
            nend--;
        nend++;
        const char *vbeg = sep;
        while (vbeg < end && (*vbeg == ':' || is_space(*vbeg)))
            vbeg++;
        char   name[512], value[512];
        size_t n = std::min((size_t)(nend - start), (size_t)511);
        memcpy(name, start, n);
        name[n] = '\0';
        n       = end > vbeg ? std::min((size_t)(end - vbeg), (size_t)511) : 0;
        memcpy(value, vbeg, n);
        value[n] = '\0';
        parse_attr(name, value);
        if (*str)
            str++;
    }
}
void Parser::parse_attribs(const char **attr) {
    for (int i = 0; attr[i]; i += 2) {
        if (strcmp(attr[i], "style") == 0)
            parse_style(attr[i + 1]);
        else
            parse_attr(attr[i], attr[i + 1]);
    }
}

const GradDef *Parser::find_grad(const char *id) const {
    for (size_t i = grads.size(); i-- > 0;)
        if (strcmp(grads[i].id, id) == 0)
            return &grads[i];
    return nullptr;
}
/* a paint from url(#id): the gradient's type and its first stop, found
   through xlink:href references when the gradient has no stops itself (the
   chain is followed at most 64 steps, where nanoSVG follows a cycle forever);
   none when neither it nor a reference has stops */
void resolve_paint(const Parser &p, const char *ref, uint8_t *type, uint32_t *color) {
    const GradDef *g = p.find_grad(ref);
    *type            = PAINT_NONE;
    if (!g)
        return;
    const GradDef *r = g;
    for (int hop = 0; r && hop < 64; hop++) {
        if (!r->stops.empty()) {
            *type  = g->type;
            *color = r->stops[0].color;
            return;
        }
        r = p.find_grad(r->ref);
    }
}

void Parser::add_shape() {
    if (plist.empty())
        return;
    const Style &a = cur();
    SvgShape     sh;
    memcpy(sh.id, a.id, sizeof(sh.id));
    sh.stroke_width = a.stroke_width * xf_avg_scale(a.xf);
    sh.opacity      = a.opacity;
    sh.visible      = a.visible;
    sh.paths.assign(plist.rbegin(), plist.rend()); /* nanoSVG prepends each path */
    plist.clear();
    memcpy(sh.bounds, sh.paths[0].bounds, sizeof(sh.bounds));
    for (size_t i = 1; i < sh.paths.size(); i++) {
        sh.bounds[0] = fminf(sh.bounds[0], sh.paths[i].bounds[0]);
        sh.bounds[1] = fminf(sh.bounds[1], sh.paths[i].bounds[1]);
        sh.bounds[2] = fmaxf(sh.bounds[2], sh.paths[i].bounds[2]);
        sh.bounds[3] = fmaxf(sh.bounds[3], sh.paths[i].bounds[3]);
    }
    if (a.has_fill == 1) {
        sh.fill_type  = PAINT_COLOR;
        sh.fill_color = a.fill_color | ((uint32_t)(a.fill_opacity * 255) << 24);
    } else if (a.has_fill == 2) {
        resolve_paint(*this, a.fill_ref, &sh.fill_type, &sh.fill_color);
    }
    if (a.has_stroke == 1) {
        sh.stroke_type  = PAINT_COLOR;
        sh.stroke_color = a.stroke_color | ((uint32_t)(a.stroke_opacity * 255) << 24);
    } else if (a.has_stroke == 2) {
        resolve_paint(*this, a.stroke_ref, &sh.stroke_type, &sh.stroke_color);
    }
    img->shapes.push_back(std::move(sh));
}

int args_per_command(char cmd) {
    switch (cmd) {
    case 'v': case 'V': case 'h': case 'H': return 1;
    case 'm': case 'M': case 'l': case 'L': case 't': case 'T': return 2;
    case 'q': case 'Q': case 's': case 'S': return 4;
    case 'c': case 'C': return 6;
    case 'a': case 'A': return 7;
    default: return 0;
    }
}
float vec_ratio(float ux, float uy, float vx, float vy) {
    return (ux * vx + uy * vy) / (sqrtf(ux * ux + uy * uy) * sqrtf(vx * vx + vy * vy));
}
float vec_angle(float ux, float uy, float vx, float vy) {
    float r = vec_ratio(ux, uy, vx, vy);
    r       = r < -1.0f ? -1.0f : (r > 1.0f ? 1.0f : r);
    return ((ux * vy < uy * vx) ? -1.0f : 1.0f) * acosf(r);
}
float sq(float x) { return x * x; }

/* elliptical arc (rx ry x-rotation large-arc sweep x y): the SVG
   implementation notes' centre parametrisation, then cubic segments of at
   most 90 degrees with handle length 4/3 (1 - cos h) / sin h */
void Parser::arc_to(float *cpx, float *cpy, const float *args, bool rel) {
    float       rx = fabsf(args[0]), ry = fabsf(args[1]);
    const float rot = args[2] / 180.0f * SVG_PI;
    const int   fa = fabsf(args[3]) > 1e-6 ? 1 : 0, fs = fabsf(args[4]) > 1e-6 ? 1 : 0;
    const float x1 = *cpx, y1 = *cpy;
    const float x2 = rel ? *cpx + args[5] : args[5], y2 = rel ? *cpy + args[6] : args[6];
    float       dx = x1 - x2, dy = y1 - y2;
    float       d  = sqrtf(dx * dx + dy * dy);
    if (d < 1e-6f || rx < 1e-6f || ry < 1e-6f) {
        line_to(x2, y2);
        *cpx = x2;
        *cpy = y2;
        return;
    }
    const float sinr = sinf(rot), cosr = cosf(rot);
    const float x1p = cosr * dx / 2.0f + sinr * dy / 2.0f;
    const float y1p = -sinr * dx / 2.0f + cosr * dy / 2.0f;
    d               = sq(x1p) / sq(rx) + sq(y1p) / sq(ry);
    if (d > 1) {
        d = sqrtf(d);
        rx *= d;
        ry *= d;
    }
    float s  = 0.0f;
    float sa = sq(rx) * sq(ry) - sq(rx) * sq(y1p) - sq(ry) * sq(x1p);
    const float sb = sq(rx) * sq(y1p) + sq(ry) * sq(x1p);
    if (sa < 0.0f)
        sa = 0.0f;
    if (sb > 0.0f)
        s = sqrtf(sa / sb);
    if (fa == fs)
        s = -s;
    const float cxp = s * rx * y1p / ry;
    const float cyp = s * -ry * x1p / rx;
    const float cx  = (x1 + x2) / 2.0f + cosr * cxp - sinr * cyp;
    const float cy  = (y1 + y2) / 2.0f + sinr * cxp + cosr * cyp;
    const float ux = (x1p - cxp) / rx, uy = (y1p - cyp) / ry;
    const float vx = (-x1p - cxp) / rx, vy = (-y1p - cyp) / ry;
    const float a1 = vec_angle(1.0f, 0.0f, ux, uy);
    float       da = vec_angle(ux, uy, vx, vy);
    if (fs == 0 && da > 0)
        da -= 2 * SVG_PI;
    else if (fs == 1 && da < 0)
        da += 2 * SVG_PI;
    const Xf    m      = Xf{{cosr, sinr, -sinr, cosr, cx, cy}};
    const int   ndivs  = (int)(fabsf(da) / (SVG_PI * 0.5f) + 1.0f);
    const float hda    = (da / (float)ndivs) / 2.0f;
    float       kappa  = fabsf(4.0f / 3.0f * (1.0f - cosf(hda)) / sinf(hda));
    if (da < 0.0f)
        kappa = -kappa;
    float px = 0, py = 0, ptx = 0, pty = 0;
    for (int i = 0; i <= ndivs; i++) {
        const float a  = a1 + da * ((float)i / (float)ndivs);
        const float ca = cosf(a), sa2 = sinf(a);
        float       x, y, tx, ty;
        xf_point(m, ca * rx, sa2 * ry, &x, &y);
        xf_vec(m, -sa2 * rx * kappa, ca * ry * kappa, &tx, &ty);
        if (i > 0)
            cubic_to(px + ptx, py + pty, x - tx, y - ty, x, y);
        px  = x;
        py  = y;
        ptx = tx;
        pty = ty;
    }
    *cpx = x2;
    *cpy = y2;
}

void Parser::parse_path(const char **attr) {
    const char *d = nullptr;
    for (int i = 0; attr[i]; i += 2) {
        if (strcmp(attr[i], "d") == 0) {
            d = attr[i + 1];
        } else {
            const char *one[4] = {attr[i], attr[i + 1], nullptr, nullptr};
            parse_attribs(one);
        }
    }
    if (d) {
        pts.clear();
        float cpx = 0, cpy = 0, cpx2 = 0, cpy2 = 0; /* current point, last control point */
        bool  closed = false;
        char  cmd    = '\0';
        float args[10];
        int   nargs = 0, rargs = 0;
        char  item[64];
        while (*d) {
            item[0] = '\0';
            if ((cmd == 'A' || cmd == 'a') && (nargs == 3 || nargs == 4))
                d = next_flag(d, item);
            if (!*item)
                d = next_item(d, item);
            if (!*item)
                break;
            if (is_num(item[0])) {
                if (nargs < 10)
                    args[nargs++] = (float)parse_double(item);
                if (nargs < rargs)
                    continue;
                const bool rel = cmd >= 'a';
                switch (cmd) {
                case 'm': case 'M':
                    cpx = rel ? cpx + args[0] : args[0];
                    cpy = rel ? cpy + args[1] : args[1];
                    move_to(cpx, cpy);
                    /* further pairs are line-tos */
                    cmd   = rel ? 'l' : 'L';
                    rargs = args_per_command(cmd);
                    cpx2 = cpx;
                    cpy2 = cpy;
                    break;
                case 'l': case 'L':
                    cpx = rel ? cpx + args[0] : args[0];
                    cpy = rel ? cpy + args[1] : args[1];
                    line_to(cpx, cpy);
                    cpx2 = cpx;
                    cpy2 = cpy;
                    break;
                case 'h': case 'H':
                    cpx = rel ? cpx + args[0] : args[0];
                    line_to(cpx, cpy);
                    cpx2 = cpx;
                    cpy2 = cpy;
                    break;
                case 'v': case 'V':
                    cpy = rel ? cpy + args[0] : args[0];
                    line_to(cpx, cpy);
                    cpx2 = cpx;
                    cpy2 = cpy;
                    break;
                case 'c': case 'C': {
                    const float ox = rel ? cpx : 0.0f, oy = rel ? cpy : 0.0f;
                    const float c1x = rel ? ox + args[0] : args[0], c1y = rel ? oy + args[1] : args[1];
                    const float c2x = rel ? ox + args[2] : args[2], c2y = rel ? oy + args[3] : args[3];
                    const float ex = rel ? ox + args[4] : args[4], ey = rel ? oy + args[5] : args[5];
                    cubic_to(c1x, c1y, c2x, c2y, ex, ey);
                    cpx2 = c2x;
                    cpy2 = c2y;
                    cpx  = ex;
                    cpy  = ey;
                    break;
                }
                case 's': case 'S': {
                    const float c2x = rel ? cpx + args[0] : args[0], c2y = rel ? cpy + args[1] : args[1];
                    const float ex = rel ? cpx + args[2] : args[2], ey = rel ? cpy + args[3] : args[3];
                    cubic_to(2 * cpx - cpx2, 2 * cpy - cpy2, c2x, c2y, ex, ey); /* reflected control point */
                    cpx2 = c2x;
                    cpy2 = c2y;
                    cpx  = ex;
                    cpy  = ey;
                    break;
                }
                case 'q': case 'Q': case 't': case 'T': {
                    const bool  smooth = cmd == 't' || cmd == 'T';
                    const float x1 = cpx, y1 = cpy;
                    float       qx, qy, ex, ey;
                    if (smooth) {
                        ex = rel ? cpx + args[0] : args[0];
                        ey = rel ? cpy + args[1] : args[1];
                        qx = 2 * x1 - cpx2;
                        qy = 2 * y1 - cpy2;
                    } else {
                        qx = rel ? cpx + args[0] : args[0];
                        qy = rel ? cpy + args[1] : args[1];
                        ex = rel ? cpx + args[2] : args[2];
                        ey = rel ? cpy + args[3] : args[3];
                    }
                    /* the quadratic as a cubic: control points 2/3 of the way to q */
                    cubic_to(x1 + 2.0f / 3.0f * (qx - x1), y1 + 2.0f / 3.0f * (qy - y1), ex + 2.0f / 3.0f * (qx - ex),
                             ey + 2.0f / 3.0f * (qy - ey), ex, ey);
                    cpx2 = qx;
                    cpy2 = qy;
                    cpx  = ex;
                    cpy  = ey;
                    break;
                }
                case 'a': case 'A':
                    arc_to(&cpx, &cpy, args, rel);
                    cpx2 = cpx;
                    cpy2 = cpy;
                    break;
                default:
                    if (nargs >= 2) {
                        cpx  = args[nargs - 2];
                        cpy  = args[nargs - 1];
                        cpx2 = cpx;
                        cpy2 = cpy;
                    }
                    break;
                }
                nargs = 0;
            } else {
                cmd   = item[0];
                rargs = args_per_command(cmd);
                if (cmd == 'M' || cmd == 'm') {
                    if (!pts.empty())
                        add_path(closed);
                    pts.clear();
                    closed = false;
                    nargs  = 0;
                } else if (cmd == 'Z' || cmd == 'z') {
                    if (!pts.empty()) {
                        cpx  = pts[0];
                        cpy  = pts[1];
                        cpx2 = cpx;
                        cpy2 = cpy;
                        add_path(true);
                    }
                    pts.clear();
                    move_to(cpx, cpy);
                    closed = false;
                    nargs  = 0;
                }
            }
        }
        if (!pts.empty())
            add_path(closed);
    }
    add_shape();
}

void Parser::parse_rect(const char **attr) {
    float x = 0, y = 0, w = 0, h = 0, rx = -1, ry = -1; /* negative radius: not given */
    for (int i = 0; attr[i]; i += 2) {
        if (parse_attr(attr[i], attr[i + 1]))
            continue;
        const char *n = attr[i], *v = attr[i + 1];
        if (strcmp(n, "x") == 0)
            x = coord(v, orig_x(), width());
        if (strcmp(n, "y") == 0)
            y = coord(v, orig_y(), height());
        if (strcmp(n, "width") == 0)
            w = coord(v, 0.0f, width());
        if (strcmp(n, "height") == 0)
            h = coord(v, 0.0f, height());
        if (strcmp(n, "rx") == 0)
            rx = fabsf(coord(v, 0.0f, width()));
        if (strcmp(n, "ry") == 0)
            ry = fabsf(coord(v, 0.0f, height()));
    }
    if (rx < 0.0f && ry > 0.0f)
        rx = ry;
    if (ry < 0.0f && rx > 0.0f)
        ry = rx;
    rx = rx < 0.0f ? 0.0f : rx;
    ry = ry < 0.0f ? 0.0f : ry;
    if (rx > w / 2.0f)
        rx = w / 2.0f;
    if (ry > h / 2.0f)
        ry = h / 2.0f;
    if (w == 0.0f || h == 0.0f)
        return;
    pts.clear();
    if (rx < 0.00001f || ry < 0.0001f) {
        move_to(x, y);
        line_to(x + w, y);
        line_to(x + w, y + h);
        line_to(x, y + h);
    } else {
        const float k = 1 - SVG_KAPPA; /* handle inset of a rounded corner */
        move_to(x + rx, y);
        line_to(x + w - rx, y);
        cubic_to(x + w - rx * k, y, x + w, y + ry * k, x + w, y + ry);
        line_to(x + w, y + h - ry);
        cubic_to(x + w, y + h - ry * k, x + w - rx * k, y + h, x + w - rx, y + h);
        line_to(x + rx, y + h);
        cubic_to(x + rx * k, y + h, x, y + h - ry * k, x, y + h - ry);
        line_to(x, y + ry);
        cubic_to(x, y + ry * k, x + rx * k, y, x + rx, y);
    }
    add_path(true);
    add_shape();
}
/* circle (r) or ellipse (rx, ry): four quarter-turn cubics from (cx + rx, cy) */
void Parser::parse_ellipse(const char **attr, bool circle) {
    float cx = 0, cy = 0, rx = 0, ry = 0;
    for (int i = 0; attr[i]; i += 2) {
        if (parse_attr(attr[i], attr[i + 1]))
            continue;
        const char *n = attr[i], *v = attr[i + 1];
        if (strcmp(n, "cx") == 0)
            cx = coord(v, orig_x(), width());
        if (strcmp(n, "cy") == 0)
            cy = coord(v, orig_y(), height());
        if (circle && strcmp(n, "r") == 0)
            rx = ry = fabsf(coord(v, 0.0f, diag()));
        if (!circle && strcmp(n, "rx") == 0)
            rx = fabsf(coord(v, 0.0f, width()));
        if (!circle && strcmp(n, "ry") == 0)
            ry = fabsf(coord(v, 0.0f, height()));
    }
    if (!(rx > 0.0f && ry > 0.0f))
        return;
    const float k = SVG_KAPPA;
    pts.clear();
    move_to(cx + rx, cy);
    cubic_to(cx + rx, cy + ry * k, cx + rx * k, cy + ry, cx, cy + ry);
    cubic_to(cx - rx * k, cy + ry, cx - rx, cy + ry * k, cx - rx, cy);
    cubic_to(cx - rx, cy - ry * k, cx - rx * k, cy - ry, cx, cy - ry);
    cubic_to(cx + rx * k, cy - ry, cx + rx, cy - ry * k, cx + rx, cy);
    add_path(true);
    add_shape();
}
void Parser::parse_line(const char **attr) {
    float x1 = 0, y1 = 0, x2 = 0, y2 = 0;
    for (int i = 0; attr[i]; i += 2) {
        if (parse_attr(attr[i], attr[i + 1]))
            continue;
        const char *n = attr[i], *v = attr[i + 1];
        if (strcmp(n, "x1") == 0)
            x1 = coord(v, orig_x(), width());
        if (strcmp(n, "y1") == 0)
            y1 = coord(v, orig_y(), height());
        if (strcmp(n, "x2") == 0)
            x2 = coord(v, orig_x(), width());
        if (strcmp(n, "y2") == 0)
            y2 = coord(v, orig_y(), height());
    }
    pts.clear();
    move_to(x1, y1);
    line_to(x2, y2);
    add_path(false);
    add_shape();
}
void Parser::parse_poly(const char **attr, bool closed) {
    pts.clear();
    for (int i = 0; attr[i]; i += 2) {
        if (parse_attr(attr[i], attr[i + 1]) || strcmp(attr[i], "points") != 0)
            continue;
        const char *s = attr[i + 1];
        float       a[2];
        int         na = 0, npts = 0;
        char        item[64];
        while (*s) {
            s       = next_item(s, item);
            a[na++] = (float)parse_double(item);
            if (na >= 2) {
                if (npts == 0)
                    move_to(a[0], a[1]);
                else
                    line_to(a[0], a[1]);
                na = 0;
                npts++;
            }
        }
    }
    add_path(closed);
    add_shape();
}
void Parser::parse_svg(const char **attr) {
    for (int i = 0; attr[i]; i += 2) {
        if (parse_attr(attr[i], attr[i + 1]))
            continue;
        const char *n = attr[i], *v = attr[i + 1];
        if (strcmp(n, "width") == 0) {
            img->width = coord(v, 0.0f, 0.0f);
        } else if (strcmp(n, "height") == 0) {
            img->height = coord(v, 0.0f, 0.0f);
        } else if (strcmp(n, "viewBox") == 0) {
            float *dst[4] = {&view_minx, &view_miny, &view_w, &view_h};
            char   buf[64];
            for (int k = 0; k < 4; k++) {
                v       = scan_number(v, buf, 64);
                *dst[k] = (float)parse_double(buf);
                while (is_space(*v) || *v == '%' || *v == ',')
                    v++;
                if (!*v && k < 3)
                    return; /* a short viewBox also ends the element's attributes */
            }
        } else if (strcmp(n, "preserveAspectRatio") == 0) {
            if (strstr(v, "none")) {
                align_type = 0;
            } else {
                if (strstr(v, "xMin"))
                    align_x = 0;
                else if (strstr(v, "xMid"))
                    align_x = 1;
                else if (strstr(v, "xMax"))
                    align_x = 2;
                if (strstr(v, "yMin"))
                    align_y = 0;
                else if (strstr(v, "yMid"))
                    align_y = 1;
                else if (strstr(v, "yMax"))
                    align_y = 2;
                align_type = strstr(v, "slice") ? 2 : 1;
            }
        }
    }
}
void Parser::parse_gradient(const char **attr, uint8_t type) {
    GradDef g;
    memset(g.id, 0, sizeof(g.id));
    memset(g.ref, 0, sizeof(g.ref));
    g.type = type;
    for (int i = 0; attr[i]; i += 2) {
        if (strcmp(attr[i], "id") == 0) {
            copy_id(g.id, attr[i + 1]);
        } else if (!parse_attr(attr[i], attr[i + 1]) && strcmp(attr[i], "xlink:href") == 0) {
            strncpy(g.ref, attr[i + 1] + 1, 62); /* past the '#' */
            g.ref[62] = '\0';
        }
    }
    grads.push_back(std::move(g));
}
/* a stop joins the most recent gradient, kept sorted by offset (a new stop
   goes before the first with a larger offset) */
void Parser::parse_stop(const char **attr) {
    Style &a       = cur();
    a.stop_offset  = 0;
    a.stop_color   = 0;
    a.stop_opacity = 1.0f;
    for (int i = 0; attr[i]; i += 2)
        parse_attr(attr[i], attr[i + 1]);
    if (grads.empty())
        return;
    std::vector<GradStop> &v = grads.back().stops;
    size_t                 k = v.size();
    for (size_t i = 0; i < v.size(); i++)
        if (a.stop_offset < v[i].offset) {
            k = i;
            break;
        }
    v.insert(v.begin() + (long)k, GradStop{a.stop_color | ((uint32_t)(a.stop_opacity * 255) << 24), a.stop_offset});
}
void Parser::start_element(const char *el, const char **attr) {
    if (in_defs) {
        if (strcmp(el, "linearGradient") == 0)
            parse_gradient(attr, PAINT_LINEAR);
        else if (strcmp(el, "radialGradient") == 0)
            parse_gradient(attr, PAINT_RADIAL);
        else if (strcmp(el, "stop") == 0)
            parse_stop(attr);
        return;
    }
    if (strcmp(el, "g") == 0) {
        push();
        parse_attribs(attr);
        return;
    }
    struct Scoped {
        Parser &p;
        explicit Scoped(Parser &q) : p(q) { p.push(); }
        ~Scoped() { p.pop(); }
    };
    if (strcmp(el, "path") == 0) {
        Scoped s(*this);
        parse_path(attr);
    } else if (strcmp(el, "rect") == 0) {
        Scoped s(*this);
        parse_rect(attr);
    } else if (strcmp(el, "circle") == 0) {
        Scoped s(*this);
        parse_ellipse(attr, true);
    } else if (strcmp(el, "ellipse") == 0) {
        Scoped s(*this);
        parse_ellipse(attr, false);
    } else if (strcmp(el, "line") == 0) {
        Scoped s(*this);
        parse_line(attr);
    } else if (strcmp(el, "polyline") == 0) {
        Scoped s(*this);
        parse_poly(attr, false);
    } else if (strcmp(el, "polygon") == 0) {
        Scoped s(*this);
        parse_poly(attr, true);
    } else if (strcmp(el, "linearGradient") == 0) {
        parse_gradient(attr, PAINT_LINEAR);
    } else if (strcmp(el, "radialGradient") == 0) {
        parse_gradient(attr, PAINT_RADIAL);
    } else if (strcmp(el, "stop") == 0) {
        parse_stop(attr);
    } else if (strcmp(el, "defs") == 0) {
        in_defs = true;
    } else if (strcmp(el, "svg") == 0) {
        parse_svg(attr);
    }
}
void Parser::end_element(const char *el) {
    if (strcmp(el, "g") == 0)
        pop();
    else if (strcmp(el, "defs") == 0)
        in_defs = false;
}

/* ---- the XML subset: text between '<' and '>' is a tag; its name runs to
   the first space; attributes are name="value" or name='value'; a tag
   starting with '/' ends an element, one whose attributes reach a '/' starts
   and ends it; '<?' and '<!' tags are skipped.  At most 127 attributes. */
void parse_tag(Parser &p, char *s) {
    const char *attr[256];
    int         na    = 0;
    bool        start = false, end = false;
    while (is_space(*s))
        s++;
    if (*s == '/') {
        s++;
        end = true;
    } else {
        start = true;
    }
    if (!*s || *s == '?' || *s == '!')
        return;
    char *name = s;
    while (*s && !is_space(*s))
        s++;
    if (*s)
        *s++ = '\0';
    while (!end && *s && na < 256 - 3) {
        while (is_space(*s))
            s++;
        if (!*s)
            break;
        if (*s == '/') {
            end = true;
            break;
        }
        char *an = s;
        while (*s && !is_space(*s) && *s != '=')
            s++;
        if (*s)
            *s++ = '\0';
        while (*s && *s != '"' && *s != '\'')
            s++;
        if (!*s)
            break;
        const char q = *s++;
        char      *av = s;
        while (*s && *s != q)
            s++;
        if (*s)
            *s++ = '\0';
        attr[na++] = an;
        attr[na++] = av;
    }
    attr[na++] = nullptr;
    attr[na++] = nullptr;
    if (start)
        p.start_element(name, attr);
    if (end)
        p.end_element(name);
}
void parse_xml(Parser &p, char *s) {
    char *mark   = s;
    bool  in_tag = false;
    for (; *s; s++) {
        if (*s == '<' && !in_tag) {
            mark   = s + 1;
            in_tag = true;
        } else if (*s == '>' && in_tag) {
            *s = '\0';
            parse_tag(p, mark);
            in_tag = false;
        }
    }
}

float view_align(float content, float container, int type) {
    if (type == 0)
        return 0;
    if (type == 2)
        return container - content;
    return (container - content) * 0.5f;
}
/* the viewBox (or, without one, the size or the drawing's bounds) onto the
   image size in the requested units; stroke widths by the mean scale */
void Parser::scale_to_viewbox(const char *units) {
    float b[4] = {0, 0, 0, 0};
    if (!img->shapes.empty()) {
        memcpy(b, img->shapes[0].bounds, sizeof(b));
        for (size_t i = 1; i < img->shapes.size(); i++) {
            const float *sb = img->shapes[i].bounds;
            b[0]            = fminf(b[0], sb[0]);
            b[1]            = fminf(b[1], sb[1]);
            b[2]            = fmaxf(b[2], sb[2]);
            b[3]            = fmaxf(b[3], sb[3]);
        }
    }
    if (view_w == 0) {
        if (img->width > 0) {
            view_w = img->width;
        } else {
            view_minx = b[0];
            view_w    = b[2] - b[0];
        }
    }
    if (view_h == 0) {
        if (img->height > 0) {
            view_h = img->height;
        } else {
            view_miny = b[1];
            view_h    = b[3] - b[1];
        }
    }
    if (img->width == 0)
        img->width = view_w;
    if (img->height == 0)
        img->height = view_h;
    float       tx = -view_minx, ty = -view_miny;
    float       sx = view_w > 0 ? img->width / view_w : 0;
    float       sy = view_h > 0 ? img->height / view_h : 0;
    const float us = 1.0f / to_px(Coord{1.0f, parse_units(units)}, 0.0f, 1.0f);
    if (align_type == 1 || align_type == 2) { /* meet / slice: one uniform scale */
        sx = sy = align_type == 1 ? fminf(sx, sy) : fmaxf(sx, sy);
        tx += view_align(view_w * sx, img->width, align_x) / sx;
        ty += view_align(view_h * sy, img->height, align_y) / sy;
    }
    sx *= us;
    sy *= us;
    const float avg = (sx + sy) / 2.0f;
    for (SvgShape &sh : img->shapes) {
        sh.bounds[0] = (sh.bounds[0] + tx) * sx;
        sh.bounds[1] = (sh.bounds[1] + ty) * sy;
        sh.bounds[2] = (sh.bounds[2] + tx) * sx;
        sh.bounds[3] = (sh.bounds[3] + ty) * sy;
        for (SvgPath &pa : sh.paths) {
            pa.bounds[0] = (pa.bounds[0] + tx) * sx;
            pa.bounds[1] = (pa.bounds[1] + ty) * sy;
            pa.bounds[2] = (pa.bounds[2] + tx) * sx;
            pa.bounds[3] = (pa.bounds[3] + ty) * sy;
            for (size_t i = 0; i < pa.pts.size(); i += 2) {
                pa.pts[i]     = (pa.pts[i] + tx) * sx;
                pa.pts[i + 1] = (pa.pts[i + 1] + ty) * sy;
            }
        }
        sh.stroke_width *= avg;
    }
}

/* nsvgParse(input, units, dpi) on a copy of the text */
_vkvg_svg_t *parse_document(const char *text, size_t len, const char *units, float dpi) {
    _vkvg_svg_t *img = new (std::nothrow) _vkvg_svg_t();
    Parser      *p   = new (std::nothrow) Parser();
    if (!img || !p) {
        delete img;
        delete p;
        return nullptr;
    }
    Style &s0 = p->st[0];
    memset(&s0, 0, sizeof(s0));
    s0.xf           = xf_identity();
    s0.opacity      = 1;
    s0.fill_opacity = s0.stroke_opacity = s0.stop_opacity = 1;
    s0.stroke_width = 1;
    s0.has_fill     = 1; /* black fill, no stroke */
    s0.visible      = true;
    p->img          = img;
    p->dpi          = dpi;
    std::vector<char> buf(text, text + len);
    buf.push_back('\0');
    buf.push_back('\x01'); /* sentinel: a scan that runs past the document stops here */
    buf.push_back('\0');
    parse_xml(*p, buf.data());
    p->scale_to_viewbox(units);
    delete p;
    return img;
}
bool read_file(const char *path, std::vector<char> &out) {
    FILE *f = path ? fopen(path, "rb") : nullptr;
    if (!f)
        return false;
    bool ok = fseek(f, 0, SEEK_END) == 0;
    long n  = ok ? ftell(f) : -1;
    ok      = ok && n >= 0 && fseek(f, 0, SEEK_SET) == 0;
    if (ok) {
        out.resize((size_t)n);
        ok = fread(out.data(), 1, (size_t)n, f) == (size_t)n;
    }
    fclose(f);
    return ok;
}
/* _svg_set_color, src/nsvg/vkvg_nsvg.c:30-36: nanoSVG's ABGR word, alpha
   times the shape's opacity */
void svg_set_color(VkvgContext ctx, uint32_t c, float alpha) {
    const float a = (c >> 24 & 255) / 255.f, b = (c >> 16 & 255) / 255.f;
    const float g = (c >> 8 & 255) / 255.f, r = (c & 255) / 255.f;
    vkvg_set_source_rgba(ctx, r, g, b, a * alpha);
}
VkvgSurface surface_from(VkvgDevice dev, _vkvg_svg_t *svg) {
    if (!svg)
        return nullptr;
    VkvgSurface surf = vkvg_surface_create(dev, (uint32_t)svg->width, (uint32_t)svg->height);
    if (vkvg_surface_status(surf)) {
        vkvg_svg_destroy(svg);
        return surf;
    }
    VkvgContext ctx = vkvg_create(surf);
    vkvg_svg_render(svg, ctx, nullptr);
    vkvg_destroy(ctx);
    vkvg_svg_destroy(svg);
    return surf;
}

} /* namespace */

extern "C" {
/* src/nsvg/vkvg_nsvg.c:72-78: documents load in px at 96 dpi */
VkvgSvg vkvg_svg_load(const char *svgFilePath) {
    std::vector<char> text;
    if (!read_file(svgFilePath, text))
        return nullptr;
    return parse_document(text.data(), text.size(), "px", 96.0f);
}
VkvgSvg vkvg_svg_load_fragment(char *svgFragment) {
    if (!svgFragment)
        return nullptr;
    return parse_document(svgFragment, strlen(svgFragment), "px", 96.0f);
}
void vkvg_svg_destroy(VkvgSvg svg) { delete svg; }
void vkvg_svg_get_dimensions(VkvgSvg svg, uint32_t *width, uint32_t *height) {
    if (!svg || !width || !height)
        return;
    *width  = (uint32_t)svg->width;
    *height = (uint32_t)svg->height;
}
/* vkvg_svg_render, src/nsvg/vkvg_nsvg.c:82-136: every shape (or those whose
   id is subId) as one path of move_to / curve_to / close_path, filled even-odd
   with its fill colour, then stroked with its stroke colour; a gradient paint
   uses its first stop's colour, a radial one changes no colour */
void vkvg_svg_render(VkvgSvg svg, VkvgContext ctx, const char *subId) {
    if (!svg || vkvg_status(ctx))
        return;
    vkvg_save(ctx);
    vkvg_set_fill_rule(ctx, VKVG_FILL_RULE_EVEN_ODD);
    vkvg_set_source_rgba(ctx, 0.0f, 0.0f, 0.0f, 1.0f);
    for (const SvgShape &sh : svg->shapes) {
        if (subId && strcmp(sh.id, subId) != 0)
            continue;
        vkvg_new_path(ctx);
        const float o = sh.opacity;
        vkvg_set_line_width(ctx, sh.stroke_width);
        for (const SvgPath &pa : sh.paths) {
            const float *p  = pa.pts.data();
            const size_t np = pa.pts.size() / 2;
            vkvg_move_to(ctx, p[0], p[1]);
            for (size_t i = 1; i < np; i += 3) {
                const float *q = p + 2 * i;
                vkvg_curve_to(ctx, q[0], q[1], q[2], q[3], q[4], q[5]);
            }
            if (pa.closed)
                vkvg_close_path(ctx);
        }
        if (sh.fill_type == PAINT_COLOR || sh.fill_type == PAINT_LINEAR)
            svg_set_color(ctx, sh.fill_color, o);
        if (sh.fill_type != PAINT_NONE) {
            if (sh.stroke_type == PAINT_NONE) {
                vkvg_fill(ctx);
                continue;
            }
            vkvg_fill_preserve(ctx);
        }
        if (sh.stroke_type == PAINT_COLOR || sh.stroke_type == PAINT_LINEAR)
            svg_set_color(ctx, sh.stroke_color, o);
        vkvg_stroke(ctx);
    }
    vkvg_restore(ctx);
}
/* src/nsvg/vkvg_nsvg.c:39-70: a surface of the document's size with the
   document drawn on it, parsed at the device's horizontal dpi; the width and
   height arguments are not used, as in vkvg */
VkvgSurface vkvg_surface_create_from_svg(VkvgDevice dev, uint32_t width, uint32_t height, const char *svgFilePath) {
    (void)width;
    (void)height;
    if (vkvg_device_status(dev))
        return nullptr;
    std::vector<char> text;
    if (!read_file(svgFilePath, text))
        return nullptr;
    return surface_from(dev, parse_document(text.data(), text.size(), "px", (float)dev->hdpi));
}
VkvgSurface vkvg_surface_create_from_svg_fragment(VkvgDevice dev, uint32_t width, uint32_t height,
                                                  char *svgFragment) {
    (void)width;
    (void)height;
    if (vkvg_device_status(dev) || !svgFragment)
        return nullptr;
    return surface_from(dev, parse_document(svgFragment, strlen(svgFragment), "px", (float)dev->hdpi));
}

/* ---- read-back of a parsed document (tests) */
uint32_t vkvg_gb300_svg_shape_count(VkvgSvg svg) { return svg ? (uint32_t)svg->shapes.size() : 0u; }
int      vkvg_gb300_svg_shape(VkvgSvg svg, uint32_t i, char *id, uint32_t *u, float *f) {
    if (!svg || i >= svg->shapes.size())
        return -1;
    const SvgShape &sh = svg->shapes[i];
    if (id)
        memcpy(id, sh.id, 64);
    if (u) {
        u[0] = sh.fill_type;
        u[1] = sh.fill_color;
        u[2] = sh.stroke_type;
        u[3] = sh.stroke_color;
        u[4] = sh.visible ? 1u : 0u;
        u[5] = (uint32_t)sh.paths.size();
    }
    if (f) {
        f[0] = sh.opacity;
        f[1] = sh.stroke_width;
        memcpy(f + 2, sh.bounds, sizeof(sh.bounds));
    }
    return 0;
}
int vkvg_gb300_svg_path(VkvgSvg svg, uint32_t shape, uint32_t path, float *pts, uint32_t cap_points, uint32_t *npts,
                        uint32_t *closed) {
    if (!svg || shape >= svg->shapes.size() || path >= svg->shapes[shape].paths.size())
        return -1;
    const SvgPath &pa = svg->shapes[shape].paths[path];
    const uint32_t n  = (uint32_t)(pa.pts.size() / 2);
    if (npts)
        *npts = n;
    if (closed)
        *closed = pa.closed ? 1u : 0u;
    if (pts)
        memcpy(pts, pa.pts.data(), (size_t)std::min(n, cap_points) * 2 * sizeof(float));
    return 0;
}
} /* extern "C" */
