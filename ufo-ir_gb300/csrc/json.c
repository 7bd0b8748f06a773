/*
 * json.c - recursive-descent JSON reader with an arena allocator.
 */
#include "json.h"

#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define JSON_MAX_DEPTH 64

typedef struct arena_block {
    struct arena_block *next;
    size_t used, cap;
    unsigned char data[];
} arena_block;

struct json_doc {
    arena_block *blocks;
    json_value *root;
};

typedef struct {
    const char *p, *end, *start;
    json_doc *doc;
    char *err;
    size_t errlen;
    int failed;
} parser;

static void *arena_alloc(json_doc *d, size_t bytes)
{
    bytes = (bytes + 15) & ~(size_t) 15;
    arena_block *b = d->blocks;
    if (!b || b->cap - b->used < bytes) {
        const size_t cap = bytes > 65536 ? bytes : 65536;
        arena_block *nb = (arena_block *) malloc(sizeof(arena_block) + cap);
        if (!nb)
            return NULL;
        nb->next = d->blocks;
        nb->used = 0;
        nb->cap = cap;
        d->blocks = nb;
        b = nb;
    }
    void *r = b->data + b->used;
    b->used += bytes;
    return r;
}

static void fail(parser *ps, const char *fmt, ...)
{
    if (ps->failed)
        return;
    ps->failed = 1;
    if (!ps->err || ps->errlen == 0)
        return;
    int line = 1, col = 1;
    for (const char *q = ps->start; q < ps->p && q < ps->end; q++) {
        if (*q == '\n') {
            line++;
            col = 1;
        } else {
            col++;
        }
    }
    char msg[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof(msg), fmt, ap);
    va_end(ap);
    snprintf(ps->err, ps->errlen, "JSON line %d, column %d: %s", line, col, msg);
}

static void skip_ws(parser *ps)
{
    while (ps->p < ps->end && (*ps->p == ' ' || *ps->p == '\t' || *ps->p == '\n' || *ps->p == '\r'))
        ps->p++;
}

static json_value *new_value(parser *ps, json_type t)
{
    json_value *v = (json_value *) arena_alloc(ps->doc, sizeof(json_value));
    if (!v) {
        fail(ps, "out of memory");
        return NULL;
    }
    memset(v, 0, sizeof(*v));
    v->type = t;
    return v;
}

static int hex4(parser *ps, unsigned *out)
{
    if (ps->end - ps->p < 4) {
        fail(ps, "truncated \\u escape");
        return -1;
    }
    unsigned v = 0;
    for (int i = 0; i < 4; i++) {
        const char c = ps->p[i];
        v <<= 4;
        if (c >= '0' && c <= '9')
            v |= (unsigned) (c - '0');
        else if (c >= 'a' && c <= 'f')
            v |= (unsigned) (c - 'a' + 10);
        else if (c >= 'A' && c <= 'F')
            v |= (unsigned) (c - 'A' + 10);
        else {
            fail(ps, "bad \\u escape");
            return -1;
        }
    }
    ps->p += 4;
    *out = v;
    return 0;
}

static size_t put_utf8(char *o, unsigned cp)
{
    if (cp < 0x80) {
        o[0] = (char) cp;
        return 1;
    }
    if (cp < 0x800) {
        o[0] = (char) (0xC0 | (cp >> 6));
        o[1] = (char) (0x80 | (cp & 0x3F));
        return 2;
    }
    if (cp < 0x10000) {
        o[0] = (char) (0xE0 | (cp >> 12));
        o[1] = (char) (0x80 | ((cp >> 6) & 0x3F));
        o[2] = (char) (0x80 | (cp & 0x3F));
        return 3;
    }
    o[0] = (char) (0xF0 | (cp >> 18));
    o[1] = (char) (0x80 | ((cp >> 12) & 0x3F));
    o[2] = (char) (0x80 | ((cp >> 6) & 0x3F));
    o[3] = (char) (0x80 | (cp & 0x3F));
    return 4;
}

/* Called with ps->p on the opening quote. */
static const char *parse_string(parser *ps)
{
    ps->p++;
    const char *q = ps->p;
    size_t n = 0;
    /* the decoded string is never longer than the raw text */
    while (q < ps->end && *q != '"') {
        if (*q == '\\')
            q++;
        q++;
        n++;
    }
    if (q >= ps->end) {
        fail(ps, "unterminated string");
        return NULL;
    }
    char *out = (char *) arena_alloc(ps->doc, (size_t) (q - ps->p) + 1);
    if (!out) {
        fail(ps, "out of memory");
        return NULL;
    }
    size_t o = 0;
    while (ps->p < ps->end && *ps->p != '"') {
        unsigned char c = (unsigned char) *ps->p;
        if (c < 0x20) {
            fail(ps, "control character in string");
            return NULL;
        }
        if (c != '\\') {
            out[o++] = (char) c;
            ps->p++;
            continue;
        }
        ps->p++;
        if (ps->p >= ps->end) {
            fail(ps, "truncated escape");
            return NULL;
        }
        const char e = *ps->p++;
        switch (e) {
        case '"': out[o++] = '"'; break;
        case '\\': out[o++] = '\\'; break;
        case '/': out[o++] = '/'; break;
        case 'b': out[o++] = '\b'; break;
        case 'f': out[o++] = '\f'; break;
        case 'n': out[o++] = '\n'; break;
        case 'r': out[o++] = '\r'; break;
        case 't': out[o++] = '\t'; break;
        case 'u': {
            unsigned cp;
            if (hex4(ps, &cp))
                return NULL;
            if (cp >= 0xD800 && cp < 0xDC00) {
                unsigned lo;
                if (ps->end - ps->p < 6 || ps->p[0] != '\\' || ps->p[1] != 'u') {
                    fail(ps, "unpaired surrogate");
                    return NULL;
                }
                ps->p += 2;
                if (hex4(ps, &lo))
                    return NULL;
                if (lo < 0xDC00 || lo >= 0xE000) {
                    fail(ps, "unpaired surrogate");
                    return NULL;
                }
                cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
            } else if (cp >= 0xDC00 && cp < 0xE000) {
                fail(ps, "unpaired surrogate");
                return NULL;
            }
            if (cp == 0) {
                fail(ps, "NUL in string");
                return NULL;
            }
            o += put_utf8(out + o, cp);
            break;
        }
        default:
            fail(ps, "bad escape \\%c", e);
            return NULL;
        }
    }
    out[o] = '\0';
    ps->p++;   /* closing quote */
    (void) n;
    return out;
}

static json_value *parse_value(parser *ps, int depth);

static int grow(parser *ps, void **arr, size_t elem, size_t *cap, size_t need)
{
    if (need <= *cap)
        return 0;
    size_t nc = *cap ? *cap * 2 : 8;
    while (nc < need)
        nc *= 2;
    void *na = arena_alloc(ps->doc, nc * elem);
    if (!na) {
        fail(ps, "out of memory");
        return -1;
    }
    if (*arr)
        memcpy(na, *arr, *cap * elem);
    *arr = na;
    *cap = nc;
    return 0;
}

static json_value *parse_object(parser *ps, int depth)
{
    json_value *v = new_value(ps, JSON_OBJECT);
    if (!v)
        return NULL;
    ps->p++;
    skip_ws(ps);
    size_t cap = 0;
    if (ps->p < ps->end && *ps->p == '}') {
        ps->p++;
        return v;
    }
    for (;;) {
        skip_ws(ps);
        if (ps->p >= ps->end || *ps->p != '"') {
            fail(ps, "expected a member name");
            return NULL;
        }
        const char *key = parse_string(ps);
        if (!key)
            return NULL;
        for (size_t i = 0; i < v->count; i++)
            if (strcmp(v->keys[i], key) == 0) {
                fail(ps, "duplicate member \"%s\"", key);
                return NULL;
            }
        skip_ws(ps);
        if (ps->p >= ps->end || *ps->p != ':') {
            fail(ps, "expected ':'");
            return NULL;
        }
        ps->p++;
        json_value *item = parse_value(ps, depth + 1);
        if (!item)
            return NULL;
        size_t kcap = cap;
        if (grow(ps, (void **) &v->keys, sizeof(char *), &kcap, v->count + 1) ||
            grow(ps, (void **) &v->items, sizeof(json_value *), &cap, v->count + 1))
            return NULL;
        v->keys[v->count] = key;
        v->items[v->count] = item;
        v->count++;
        skip_ws(ps);
        if (ps->p < ps->end && *ps->p == ',') {
            ps->p++;
            continue;
        }
        if (ps->p < ps->end && *ps->p == '}') {
            ps->p++;
            return v;
        }
        fail(ps, "expected ',' or '}'");
        return NULL;
    }
}

static json_value *parse_array(parser *ps, int depth)
{
    json_value *v = new_value(ps, JSON_ARRAY);
    if (!v)
        return NULL;
    ps->p++;
    skip_ws(ps);
    size_t cap = 0;
    if (ps->p < ps->end && *ps->p == ']') {
        ps->p++;
        return v;
    }
    for (;;) {
        json_value *item = parse_value(ps, depth + 1);
        if (!item)
            return NULL;
        if (grow(ps, (void **) &v->items, sizeof(json_value *), &cap, v->count + 1))
            return NULL;
        v->items[v->count++] = item;
        skip_ws(ps);
        if (ps->p < ps->end && *ps->p == ',') {
            ps->p++;
            continue;
        }
        if (ps->p < ps->end && *ps->p == ']') {
            ps->p++;
            return v;
        }
        fail(ps, "expected ',' or ']'");
        return NULL;
    }
}

static json_value *parse_number(parser *ps)
{
    const char *s = ps->p;
    const char *q = s;
    if (q < ps->end && *q == '-')
        q++;
    if (q >= ps->end || !(*q >= '0' && *q <= '9')) {
        fail(ps, "bad number");
        return NULL;
    }
    if (*q == '0') {
        q++;
    } else {
        while (q < ps->end && *q >= '0' && *q <= '9')
            q++;
    }
    if (q < ps->end && *q == '.') {
        q++;
        if (q >= ps->end || !(*q >= '0' && *q <= '9')) {
            fail(ps, "bad number");
            return NULL;
        }
        while (q < ps->end && *q >= '0' && *q <= '9')
            q++;
    }
    if (q < ps->end && (*q == 'e' || *q == 'E')) {
        q++;
        if (q < ps->end && (*q == '+' || *q == '-'))
            q++;
        if (q >= ps->end || !(*q >= '0' && *q <= '9')) {
            fail(ps, "bad number");
            return NULL;
        }
        while (q < ps->end && *q >= '0' && *q <= '9')
            q++;
    }
    char buf[64];
    const size_t len = (size_t) (q - s);
    if (len >= sizeof(buf)) {
        fail(ps, "number too long");
        return NULL;
    }
    memcpy(buf, s, len);
    buf[len] = '\0';
    json_value *v = new_value(ps, JSON_NUMBER);
    if (!v)
        return NULL;
    v->number = strtod(buf, NULL);
    ps->p = q;
    return v;
}

static int literal(parser *ps, const char *word)
{
    const size_t n = strlen(word);
    if ((size_t) (ps->end - ps->p) >= n && memcmp(ps->p, word, n) == 0) {
        ps->p += n;
        return 1;
    }
    return 0;
}

static json_value *parse_value(parser *ps, int depth)
{
    if (depth > JSON_MAX_DEPTH) {
        fail(ps, "nesting deeper than %d", JSON_MAX_DEPTH);
        return NULL;
    }
    skip_ws(ps);
    if (ps->p >= ps->end) {
        fail(ps, "unexpected end of input");
        return NULL;
    }
    const char c = *ps->p;
    if (c == '{')
        return parse_object(ps, depth);
    if (c == '[')
        return parse_array(ps, depth);
    if (c == '"') {
        const char *str = parse_string(ps);
        if (!str)
            return NULL;
        json_value *v = new_value(ps, JSON_STRING);
        if (v)
            v->string = str;
        return v;
    }
    if (c == '-' || (c >= '0' && c <= '9'))
        return parse_number(ps);
    if (literal(ps, "true")) {
        json_value *v = new_value(ps, JSON_BOOL);
        if (v)
            v->number = 1.0;
        return v;
    }
    if (literal(ps, "false"))
        return new_value(ps, JSON_BOOL);
    if (literal(ps, "null"))
        return new_value(ps, JSON_NULL);
    fail(ps, "unexpected character '%c'", c);
    return NULL;
}

json_doc *json_parse(const char *text, size_t len, char *err, size_t errlen)
{
    if (err && errlen)
        err[0] = '\0';
    json_doc *d = (json_doc *) calloc(1, sizeof(json_doc));
    if (!d) {
        if (err && errlen)
            snprintf(err, errlen, "out of memory");
        return NULL;
    }
    parser ps = {text, text + len, text, d, err, errlen, 0};
    d->root = text ? parse_value(&ps, 0) : NULL;
    if (d->root) {
        skip_ws(&ps);
        if (ps.p != ps.end)
            fail(&ps, "trailing characters after the document");
    } else if (!text) {
        fail(&ps, "no text");
    }
    if (ps.failed || !d->root) {
        json_free(d);
        return NULL;
    }
    return d;
}

const json_value *json_root(const json_doc *doc)
{
    return doc ? doc->root : NULL;
}

void json_free(json_doc *doc)
{
    if (!doc)
        return;
    arena_block *b = doc->blocks;
    while (b) {
        arena_block *n = b->next;
        free(b);
        b = n;
    }
    free(doc);
}

const json_value *json_get(const json_value *obj, const char *key)
{
    if (!obj || obj->type != JSON_OBJECT)
        return NULL;
    for (size_t i = 0; i < obj->count; i++)
        if (strcmp(obj->keys[i], key) == 0)
            return obj->items[i];
    return NULL;
}
