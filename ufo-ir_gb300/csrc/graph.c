/*
 * graph.c - reconstruction graphs in ufo-core's JSON format: a read node,
 * one ufo-ir method node with its projector (and ASD-POCS's df_minimizer),
 * and a write node (the layout of json-sample.json:1-43). The properties
 * are those of the plugins (src/core/ufo-ir-method-task.c:75-86,
 * src/core/ufo-ir-projector-task.c:60-93, src/core/ufo-ir-state-dependent-
 * task.c:75-80, src/tasks/ufo-ir-parallel-projector-task.c:123-137,
 * src/tasks/ufo-ir-sart-task.c:76-81, src/tasks/ufo-ir-sirt-task.c:73-77,
 * src/tasks/ufo-ir-asdpocs-task.c:104-158, src/tasks/ufo-ir-sbtv-task.c:90-101)
 * with the same ranges; GObject treats '-' and '_' in names alike.
 */
#include "ufoir.h"

#include <ctype.h>
#include <float.h>
#include <glob.h>
#include <limits.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "host.h"
#include "json.h"

typedef struct {
    char *err;
    size_t errlen;
} gctx;

static int gfail(gctx *g, int status, const char *fmt, ...)
{
    if (g->err && g->errlen) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(g->err, g->errlen, fmt, ap);
        va_end(ap);
    }
    return status;
}

/* property name with '_' read as '-' */
static int name_is(const char *key, const char *canon)
{
    for (; *key && *canon; key++, canon++) {
        const char a = *key == '_' ? '-' : *key;
        if (a != *canon)
            return 0;
    }
    return *key == '\0' && *canon == '\0';
}

static int get_uint(gctx *g, const char *node, const char *key, const json_value *v, unsigned int lo,
                    unsigned int hi, unsigned int *out)
{
    if (v->type != JSON_NUMBER || v->number != (double) (long long) v->number || v->number < (double) lo ||
        v->number > (double) hi)
        return gfail(g, UFOIR_ERR_INVALID, "%s: \"%s\" must be an integer in [%u, %u]", node, key, lo, hi);
    *out = (unsigned int) v->number;
    return UFOIR_OK;
}

static int get_float(gctx *g, const char *node, const char *key, const json_value *v, double lo, double hi,
                     float *out)
{
    if (v->type != JSON_NUMBER || !(v->number >= lo && v->number <= hi))
        return gfail(g, UFOIR_ERR_INVALID, "%s: \"%s\" must be a number in [%g, %g]", node, key, lo, hi);
    *out = (float) v->number;
    return UFOIR_OK;
}

static int get_bool(gctx *g, const char *node, const char *key, const json_value *v, int *out)
{
    if (v->type != JSON_BOOL)
        return gfail(g, UFOIR_ERR_INVALID, "%s: \"%s\" must be true or false", node, key);
    *out = v->number != 0.0;
    return UFOIR_OK;
}

static int get_string(gctx *g, const char *node, const char *key, const json_value *v, char *out, size_t cap)
{
    if (v->type != JSON_STRING || strlen(v->string) >= cap)
        return gfail(g, UFOIR_ERR_INVALID, "%s: \"%s\" must be a string shorter than %zu bytes", node, key, cap);
    strcpy(out, v->string);
    return UFOIR_OK;
}

/* plugin / package of a node object */
static int node_header(gctx *g, const json_value *n, const char **plugin, const char **package, const char **name,
                       const json_value **props)
{
    if (!n || n->type != JSON_OBJECT)
        return gfail(g, UFOIR_ERR_INVALID, "a node must be an object");
    const json_value *pl = json_get(n, "plugin"), *pk = json_get(n, "package"), *nm = json_get(n, "name");
    if (!pl || pl->type != JSON_STRING)
        return gfail(g, UFOIR_ERR_INVALID, "a node without a \"plugin\" string");
    if (pk && pk->type != JSON_STRING)
        return gfail(g, UFOIR_ERR_INVALID, "node \"%s\": \"package\" must be a string", pl->string);
    if (nm && nm->type != JSON_STRING)
        return gfail(g, UFOIR_ERR_INVALID, "node \"%s\": \"name\" must be a string", pl->string);
    for (size_t i = 0; i < n->count; i++) {
        const char *k = n->keys[i];
        if (strcmp(k, "plugin") && strcmp(k, "package") && strcmp(k, "name") && strcmp(k, "properties"))
            return gfail(g, UFOIR_ERR_INVALID, "node \"%s\": unknown member \"%s\"", pl->string, k);
    }
    *plugin = pl->string;
    *package = pk ? pk->string : NULL;
    *name = nm ? nm->string : pl->string;
    *props = json_get(n, "properties");
    if (*props && (*props)->type != JSON_OBJECT)
        return gfail(g, UFOIR_ERR_INVALID, "node \"%s\": \"properties\" must be an object", pl->string);
    return UFOIR_OK;
}

static int is_ir(const char *package)
{
    return package && strcmp(package, "ir") == 0;
}

static int parse_projector(gctx *g, const json_value *n, ufoir_projector_params *p)
{
    const char *plugin, *package, *name;
    const json_value *props;
    int rc = node_header(g, n, &plugin, &package, &name, &props);
    if (rc)
        return rc;
    if (strcmp(plugin, "parallel-projector") != 0 || !is_ir(package))
        return gfail(g, UFOIR_ERR_UNSUPPORTED, "projector \"%s\" (package %s): only \"parallel-projector\" of "
                     "package \"ir\" exists", plugin, package ? package : "none");
    ufoir_projector_params_init(p);
    for (size_t i = 0; props && i < props->count && rc == UFOIR_OK; i++) {
        const char *k = props->keys[i];
        const json_value *v = props->items[i];
        if (name_is(k, "model"))
            rc = get_string(g, name, k, v, p->model, sizeof(p->model));
        else if (name_is(k, "angles-num"))
            rc = get_uint(g, name, k, v, 0, UINT_MAX, &p->angles_num);
        else if (name_is(k, "is-forward"))
            rc = get_bool(g, name, k, v, &p->is_forward);
        else if (name_is(k, "axis-position"))
            rc = get_float(g, name, k, v, -1.0, FLT_MAX, &p->axis_position);
        else if (name_is(k, "step"))
            rc = get_float(g, name, k, v, 0.0, FLT_MAX, &p->step);
        else if (name_is(k, "relaxation"))
            rc = get_float(g, name, k, v, -FLT_MAX, FLT_MAX, &p->relaxation);
        else if (name_is(k, "correction-scale"))
            rc = get_float(g, name, k, v, -FLT_MAX, FLT_MAX, &p->correction_scale);
        else if (name_is(k, "arithmetic")) {
            /* extension: the tiled projectors' interpolation arithmetic */
            if (v->type == JSON_STRING && strcmp(v->string, "exact") == 0)
                p->arithmetic = UFOIR_ARITH_EXACT;
            else if (v->type == JSON_STRING && strcmp(v->string, "fast") == 0)
                p->arithmetic = UFOIR_ARITH_FAST;
            else
                rc = gfail(g, UFOIR_ERR_INVALID, "%s: \"arithmetic\" must be \"exact\" or \"fast\"", name);
        } else
            rc = gfail(g, UFOIR_ERR_INVALID, "%s: no property \"%s\"", name, k);
    }
    return rc;
}

static int parse_norm_mode(gctx *g, const char *node, const char *k, const json_value *v, int *mode)
{
    if (v->type == JSON_STRING && strcmp(v->string, "compat") == 0)
        *mode = UFOIR_NORM_COMPAT;
    else if (v->type == JSON_STRING && strcmp(v->string, "fp64") == 0)
        *mode = UFOIR_NORM_FP64;
    else
        return gfail(g, UFOIR_ERR_INVALID, "%s: \"%s\" must be \"compat\" or \"fp64\"", node, k);
    return UFOIR_OK;
}

/* SART node properties (also the df_minimizer of ASD-POCS) */
static int parse_sart_props(gctx *g, const char *name, const json_value *props, ufoir_sart_params *s,
                            ufoir_projector_params *proj, int *have_proj, int allow_projector)
{
    int rc = UFOIR_OK;
    for (size_t i = 0; props && i < props->count && rc == UFOIR_OK; i++) {
        const char *k = props->keys[i];
        const json_value *v = props->items[i];
        if (name_is(k, "num-iterations"))
            rc = get_uint(g, name, k, v, 1, UINT_MAX, &s->num_iterations);
        else if (name_is(k, "relaxation-factor"))
            rc = get_float(g, name, k, v, 0.0, 1.0, &s->relaxation_factor);
        else if (name_is(k, "projector") && allow_projector) {
            rc = parse_projector(g, v, proj);
            *have_proj = 1;
        } else if (name_is(k, "projector"))
            rc = gfail(g, UFOIR_ERR_INVALID, "%s: the df_minimizer uses the method's projector", name);
        else
            rc = gfail(g, UFOIR_ERR_INVALID, "%s: no property \"%s\"", name, k);
    }
    return rc;
}

static int parse_method(gctx *g, const json_value *n, ufoir_graph *out)
{
    const char *plugin, *package, *name;
    const json_value *props;
    int rc = node_header(g, n, &plugin, &package, &name, &props);
    if (rc)
        return rc;
    int have_proj = 0;
    if (strcmp(plugin, "sart") == 0 || strcmp(plugin, "sirt") == 0) {
        out->method = plugin[1] == 'a' ? UFOIR_METHOD_SART : UFOIR_METHOD_SIRT;
        rc = parse_sart_props(g, name, props, &out->sart, &out->projector, &have_proj, 1);
    } else if (strcmp(plugin, "asdpocs") == 0) {
        out->method = UFOIR_METHOD_ASDPOCS;
        ufoir_asdpocs_params *a = &out->asdpocs;
        for (size_t i = 0; props && i < props->count && rc == UFOIR_OK; i++) {
            const char *k = props->keys[i];
            const json_value *v = props->items[i];
            if (name_is(k, "num-iterations"))
                rc = get_uint(g, name, k, v, 1, UINT_MAX, &a->num_iterations);
            else if (name_is(k, "beta"))
                rc = get_float(g, name, k, v, 0.0, FLT_MAX, &a->beta);
            else if (name_is(k, "beta-red"))
                rc = get_float(g, name, k, v, 0.0, FLT_MAX, &a->beta_red);
            else if (name_is(k, "alpha"))
                rc = get_float(g, name, k, v, 0.0, FLT_MAX, &a->alpha);
            else if (name_is(k, "alpha-red"))
                rc = get_float(g, name, k, v, 0.0, FLT_MAX, &a->alpha_red);
            else if (name_is(k, "r-max"))
                rc = get_float(g, name, k, v, 0.0, FLT_MAX, &a->r_max);
            else if (name_is(k, "ng"))
                rc = get_uint(g, name, k, v, 0, 1000, &a->ng);
            else if (name_is(k, "positive-constraint"))
                rc = get_bool(g, name, k, v, &a->positive_constraint);
            else if (name_is(k, "norm-mode"))
                rc = parse_norm_mode(g, name, k, v, &a->norm_mode);
            else if (name_is(k, "projector")) {
                rc = parse_projector(g, v, &out->projector);
                have_proj = 1;
            } else if (name_is(k, "df-minimizer")) {
                const char *pl2, *pk2, *nm2;
                const json_value *pr2;
                rc = node_header(g, v, &pl2, &pk2, &nm2, &pr2);
                if (!rc && (strcmp(pl2, "sart") != 0 || !is_ir(pk2)))
                    rc = gfail(g, UFOIR_ERR_UNSUPPORTED, "%s: df_minimizer \"%s\" (only \"sart\" of package "
                               "\"ir\")", name, pl2);
                if (!rc)
                    rc = parse_sart_props(g, nm2, pr2, &a->df_minimizer, NULL, NULL, 0);
            } else {
                rc = gfail(g, UFOIR_ERR_INVALID, "%s: no property \"%s\"", name, k);
            }
        }
    } else if (strcmp(plugin, "sbtv") == 0) {
        out->method = UFOIR_METHOD_SBTV;
        ufoir_sbtv_params *b = &out->sbtv;
        for (size_t i = 0; props && i < props->count && rc == UFOIR_OK; i++) {
            const char *k = props->keys[i];
            const json_value *v = props->items[i];
            if (name_is(k, "num-iterations"))
                rc = get_uint(g, name, k, v, 1, UINT_MAX, &b->num_iterations);
            else if (name_is(k, "lambda"))
                rc = get_float(g, name, k, v, 0.0, FLT_MAX, &b->lambda);
            else if (name_is(k, "mu"))
                rc = get_float(g, name, k, v, 0.0, FLT_MAX, &b->mu);
            else if (name_is(k, "norm-mode"))
                rc = parse_norm_mode(g, name, k, v, &b->norm_mode);
            else if (name_is(k, "projector")) {
                rc = parse_projector(g, v, &out->projector);
                have_proj = 1;
            } else
                rc = gfail(g, UFOIR_ERR_INVALID, "%s: no property \"%s\"", name, k);
        }
    } else {
        return gfail(g, UFOIR_ERR_UNSUPPORTED, "plugin \"%s\" is not a ufo-ir method", plugin);
    }
    if (rc)
        return rc;
    if (!is_ir(package))
        return gfail(g, UFOIR_ERR_INVALID, "method \"%s\" must have \"package\": \"ir\"", name);
    if (!have_proj)
        return gfail(g, UFOIR_ERR_INVALID, "method \"%s\" has no \"projector\"", name);
    return UFOIR_OK;
}

static int parse_read(gctx *g, const json_value *props, const char *name, ufoir_graph *out)
{
    int rc = UFOIR_OK;
    unsigned int bitdepth = 32;
    for (size_t i = 0; props && i < props->count && rc == UFOIR_OK; i++) {
        const char *k = props->keys[i];
        const json_value *v = props->items[i];
        if (name_is(k, "path"))
            rc = get_string(g, name, k, v, out->read_path, sizeof(out->read_path));
        else if (name_is(k, "raw-width"))
            rc = get_uint(g, name, k, v, 1, UINT_MAX, &out->read_raw_width);
        else if (name_is(k, "raw-height"))
            rc = get_uint(g, name, k, v, 1, UINT_MAX, &out->read_raw_height);
        else if (name_is(k, "raw-offset")) {
            unsigned int off = 0;
            rc = get_uint(g, name, k, v, 0, UINT_MAX, &off);
            out->read_raw_offset = off;
        } else if (name_is(k, "raw-bitdepth"))
            rc = get_uint(g, name, k, v, 32, 32, &bitdepth);
        else
            rc = gfail(g, UFOIR_ERR_UNSUPPORTED, "%s: property \"%s\" is not supported (path, raw-width, "
                       "raw-height, raw-offset, raw-bitdepth 32)", name, k);
    }
    if (!rc && out->read_path[0] == '\0')
        rc = gfail(g, UFOIR_ERR_INVALID, "%s: no \"path\"", name);
    if (!rc && (out->read_raw_width == 0) != (out->read_raw_height == 0))
        rc = gfail(g, UFOIR_ERR_INVALID, "%s: raw-width and raw-height go together", name);
    return rc;
}

static int parse_write(gctx *g, const json_value *props, const char *name, ufoir_graph *out)
{
    int rc = UFOIR_OK;
    unsigned int bits = 32;
    for (size_t i = 0; props && i < props->count && rc == UFOIR_OK; i++) {
        const char *k = props->keys[i];
        const json_value *v = props->items[i];
        if (name_is(k, "filename"))
            rc = get_string(g, name, k, v, out->write_filename, sizeof(out->write_filename));
        else if (name_is(k, "bits"))
            rc = get_uint(g, name, k, v, 32, 32, &bits);
        else
            rc = gfail(g, UFOIR_ERR_UNSUPPORTED, "%s: property \"%s\" is not supported (filename, bits 32)", name, k);
    }
    if (!rc && out->write_filename[0] == '\0')
        rc = gfail(g, UFOIR_ERR_INVALID, "%s: no \"filename\"", name);
    return rc;
}

int ufoir_graph_parse(const char *json, size_t len, ufoir_graph *out, char *err, size_t errlen)
{
    gctx g = {err, errlen};
    if (err && errlen)
        err[0] = '\0';
    if (!json || !out)
        return gfail(&g, UFOIR_ERR_INVALID, "no text or output");
    memset(out, 0, sizeof(*out));
    out->method = -1;
    ufoir_projector_params_init(&out->projector);
    ufoir_sart_params_init(&out->sart);
    ufoir_asdpocs_params_init(&out->asdpocs);
    ufoir_sbtv_params_init(&out->sbtv);
    char jerr[256];
    json_doc *doc = json_parse(json, len, jerr, sizeof(jerr));
    if (!doc)
        return gfail(&g, UFOIR_ERR_IO, "%s", jerr);
    const json_value *root = json_root(doc);
    int rc = UFOIR_OK;
    const json_value *nodes = json_get(root, "nodes"), *edges = json_get(root, "edges");
    const char *read_name = NULL, *method_name = NULL, *write_name = NULL;
    if (root->type != JSON_OBJECT || !nodes || nodes->type != JSON_ARRAY)
        rc = gfail(&g, UFOIR_ERR_INVALID, "the document must be an object with a \"nodes\" array");
    for (size_t i = 0; root->type == JSON_OBJECT && i < root->count && rc == UFOIR_OK; i++)
        if (strcmp(root->keys[i], "nodes") && strcmp(root->keys[i], "edges"))
            rc = gfail(&g, UFOIR_ERR_INVALID, "unknown member \"%s\" (nodes, edges)", root->keys[i]);
    for (size_t i = 0; rc == UFOIR_OK && i < nodes->count; i++) {
        const char *plugin, *package, *name;
        const json_value *props;
        rc = node_header(&g, nodes->items[i], &plugin, &package, &name, &props);
        if (rc)
            break;
        for (size_t j = 0; j < i; j++) {
            const json_value *nm = json_get(nodes->items[j], "name"), *pl = json_get(nodes->items[j], "plugin");
            const char *other = nm ? nm->string : pl->string;
            if (strcmp(other, name) == 0)
                rc = gfail(&g, UFOIR_ERR_INVALID, "two nodes named \"%s\"", name);
        }
        if (rc)
            break;
        if (strcmp(plugin, "read") == 0 && !package) {
            if (read_name)
                rc = gfail(&g, UFOIR_ERR_UNSUPPORTED, "more than one read node");
            else {
                read_name = name;
                rc = parse_read(&g, props, name, out);
            }
        } else if (strcmp(plugin, "write") == 0 && !package) {
            if (write_name)
                rc = gfail(&g, UFOIR_ERR_UNSUPPORTED, "more than one write node");
            else {
                write_name = name;
                rc = parse_write(&g, props, name, out);
            }
        } else if (is_ir(package)) {
            if (method_name)
                rc = gfail(&g, UFOIR_ERR_UNSUPPORTED, "more than one ufo-ir method node");
            else {
                method_name = name;
                rc = parse_method(&g, nodes->items[i], out);
            }
        } else {
            rc = gfail(&g, UFOIR_ERR_UNSUPPORTED, "plugin \"%s\" is not supported (read, write, ufo-ir methods)",
                       plugin);
        }
    }
    if (rc == UFOIR_OK && !method_name)
        rc = gfail(&g, UFOIR_ERR_INVALID, "no ufo-ir method node");
    /* edges: read -> method -> write, as far as those nodes exist */
    if (rc == UFOIR_OK && edges) {
        if (edges->type != JSON_ARRAY)
            rc = gfail(&g, UFOIR_ERR_INVALID, "\"edges\" must be an array");
        int seen_in = 0, seen_out = 0;
        for (size_t i = 0; rc == UFOIR_OK && i < edges->count; i++) {
            const json_value *e = edges->items[i];
            const json_value *from = json_get(e, "from"), *to = json_get(e, "to");
            const json_value *fn = json_get(from, "name"), *tn = json_get(to, "name");
            if (!fn || !tn || fn->type != JSON_STRING || tn->type != JSON_STRING) {
                rc = gfail(&g, UFOIR_ERR_INVALID, "edge %zu: \"from\" and \"to\" need a \"name\"", i);
                break;
            }
            const json_value *port = json_get(to, "input");
            if (port && (port->type != JSON_NUMBER || port->number != 0.0)) {
                rc = gfail(&g, UFOIR_ERR_INVALID, "edge %zu: the nodes have one input (input 0)", i);
                break;
            }
            if (read_name && strcmp(fn->string, read_name) == 0 && strcmp(tn->string, method_name) == 0)
                seen_in = 1;
            else if (write_name && strcmp(fn->string, method_name) == 0 && strcmp(tn->string, write_name) == 0)
                seen_out = 1;
            else
                rc = gfail(&g, UFOIR_ERR_UNSUPPORTED, "edge %s -> %s: only read -> method -> write is supported",
                           fn->string, tn->string);
        }
        if (rc == UFOIR_OK && ((read_name && !seen_in) || (write_name && !seen_out)))
            rc = gfail(&g, UFOIR_ERR_INVALID, "the edges must join read -> %s -> write", method_name);
    }
    json_free(doc);
    return rc;
}

int ufoir_graph_load(const char *path, ufoir_graph *out, char *err, size_t errlen)
{
    gctx g = {err, errlen};
    if (!path)
        return gfail(&g, UFOIR_ERR_INVALID, "no path");
    FILE *f = fopen(path, "rb");
    if (!f)
        return gfail(&g, UFOIR_ERR_IO, "%s: cannot open", path);
    char *text = NULL;
    size_t len = 0, cap = 0;
    for (;;) {
        if (cap - len < 65536) {
            cap = cap ? 2 * cap : 65536;
            if (cap > ((size_t) 64 << 20)) {
                free(text);
                fclose(f);
                return gfail(&g, UFOIR_ERR_IO, "%s: larger than 64 MiB", path);
            }
            char *nt = (char *) realloc(text, cap);
            if (!nt) {
                free(text);
                fclose(f);
                return gfail(&g, UFOIR_ERR_NOMEM, "out of host memory");
            }
            text = nt;
        }
        const size_t got = fread(text + len, 1, cap - len, f);
        len += got;
        if (got == 0)
            break;
    }
    fclose(f);
    const int rc = ufoir_graph_parse(text, len, out, err, errlen);
    free(text);
    return rc;
}

int ufoir_graph_job_desc(const ufoir_graph *g, unsigned int n_dets, unsigned int n_angles, ufoir_job_desc *out)
{
    if (!g || !out || n_dets == 0 || n_angles == 0)
        return UFOIR_ERR_INVALID;
    if (g->method != UFOIR_METHOD_SART && g->method != UFOIR_METHOD_SIRT && g->method != UFOIR_METHOD_ASDPOCS)
        return UFOIR_ERR_UNSUPPORTED;
    if (g->projector.angles_num && g->projector.angles_num != n_angles)
        return UFOIR_ERR_INVALID;
    ufoir_job_desc_init(out);
    out->method = g->method;
    out->n_dets = n_dets;
    out->n_angles = n_angles;
    out->step = g->projector.step;
    out->axis_position = g->projector.axis_position;
    out->sart = g->sart;
    out->asdpocs = g->asdpocs;
    return UFOIR_OK;
}

/* ----------------------------------------------------------------- runner */

/* A write filename with one printf integer conversion (%d, %i, %u with an
 * optional zero flag and width) and no other '%' except "%%". */
static int counter_format(const char *fmt)
{
    int conversions = 0;
    for (const char *p = fmt; *p; p++) {
        if (*p != '%')
            continue;
        p++;
        if (*p == '%')
            continue;
        if (*p == '0')
            p++;
        while (isdigit((unsigned char) *p))
            p++;
        if (*p != 'd' && *p != 'i' && *p != 'u')
            return -1;
        conversions++;
    }
    return conversions <= 1 ? conversions : -1;
}

typedef struct {
    char **paths;
    size_t n;
    int globbed;
    glob_t gl;
    char *single[1];
} input_files;

/* A read path is a file or a glob pattern (matches in sorted order). */
static int list_inputs(ufoir_ctx *ctx, const char *pattern, input_files *in)
{
    memset(in, 0, sizeof(*in));
    if (strpbrk(pattern, "*?[")) {
        const int r = glob(pattern, 0, NULL, &in->gl);
        if (r != 0 || in->gl.gl_pathc == 0) {
            if (r == 0)
                globfree(&in->gl);
            return ufoir__fail(ctx, UFOIR_ERR_IO, "read: no file matches \"%s\"", pattern);
        }
        in->globbed = 1;
        in->paths = in->gl.gl_pathv;
        in->n = in->gl.gl_pathc;
        return UFOIR_OK;
    }
    in->single[0] = (char *) pattern;
    in->paths = in->single;
    in->n = 1;
    return UFOIR_OK;
}

static void free_inputs(input_files *in)
{
    if (in->globbed)
        globfree(&in->gl);
}

/* sinogram slices: [count][height][width] floats, appended to *buf */
static int read_all(ufoir_ctx *ctx, const ufoir_graph *g, float **buf, size_t *n_slices, unsigned int *width,
                    unsigned int *height)
{
    input_files in;
    int rc = list_inputs(ctx, g->read_path, &in);
    if (rc)
        return rc;
    *buf = NULL;
    *n_slices = 0;
    *width = *height = 0;
    size_t cap = 0;
    for (size_t f = 0; f < in.n && rc == UFOIR_OK; f++) {
        const char *path = in.paths[f];
        unsigned int w, h, pages;
        uint64_t offset = 0;
        if (g->read_raw_width) {
            w = g->read_raw_width;
            h = g->read_raw_height;
            FILE *fp = fopen(path, "rb");
            long size = -1;
            if (fp && fseek(fp, 0, SEEK_END) == 0)
                size = ftell(fp);
            if (fp)
                fclose(fp);
            const uint64_t slice_bytes = (uint64_t) w * h * 4;
            if (size < 0 || (uint64_t) size < g->read_raw_offset + slice_bytes) {
                rc = ufoir__fail(ctx, UFOIR_ERR_IO, "read: %s holds no %ux%u float32 slice at offset %llu", path, w,
                                 h, (unsigned long long) g->read_raw_offset);
                break;
            }
            pages = (unsigned int) (((uint64_t) size - g->read_raw_offset) / slice_bytes);
            offset = g->read_raw_offset;
        } else if ((rc = ufoir_io_tiff_info(path, &w, &h, &pages))) {
            ufoir__fail(ctx, rc, "read: %s", ufoir_io_last_error());
            break;
        }
        if (*n_slices && (w != *width || h != *height)) {
            rc = ufoir__fail(ctx, UFOIR_ERR_INVALID, "read: %s is %ux%u, earlier slices are %ux%u", path, w, h,
                             *width, *height);
            break;
        }
        *width = w;
        *height = h;
        const size_t per = (size_t) w * h;
        if (*n_slices + pages > cap) {
            size_t nc = cap ? 2 * cap : 16;
            while (nc < *n_slices + pages)
                nc *= 2;
            float *nb = (float *) realloc(*buf, nc * per * sizeof(float));
            if (!nb) {
                rc = ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
                break;
            }
            *buf = nb;
            cap = nc;
        }
        for (unsigned int p = 0; p < pages && rc == UFOIR_OK; p++) {
            float *dst = *buf + (*n_slices) * per;
            rc = g->read_raw_width ? ufoir_io_read_raw(path, offset + (uint64_t) p * per * 4, dst, per)
                                   : ufoir_io_read_tiff(path, p, dst, per);
            if (rc)
                ufoir__fail(ctx, rc, "read: %s", ufoir_io_last_error());
            else
                (*n_slices)++;
        }
    }
    free_inputs(&in);
    if (rc == UFOIR_OK && *n_slices == 0)
        rc = ufoir__fail(ctx, UFOIR_ERR_IO, "read: no slices in \"%s\"", g->read_path);
    if (rc) {
        free(*buf);
        *buf = NULL;
    }
    return rc;
}

static int write_all(ufoir_ctx *ctx, const ufoir_graph *g, const float *vol, size_t n_slices, unsigned int n)
{
    const int conv = counter_format(g->write_filename);
    if (conv < 0)
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "write: \"%s\" must hold at most one %%d/%%i/%%u counter",
                           g->write_filename);
    const size_t per = (size_t) n * n;
    const size_t len = strlen(g->write_filename);
    const int raw = len > 4 && strcmp(g->write_filename + len - 4, ".raw") == 0;
    int rc = UFOIR_OK;
    if (conv == 0) {
        rc = raw ? ufoir_io_write_raw(g->write_filename, vol, per * n_slices)
                 : ufoir_io_write_tiff(g->write_filename, vol, n, n, (unsigned int) n_slices);
        if (rc)
            ufoir__fail(ctx, rc, "write: %s", ufoir_io_last_error());
        return rc;
    }
    for (size_t i = 0; i < n_slices && rc == UFOIR_OK; i++) {
        char path[UFOIR_PATH_MAX + 32];
        snprintf(path, sizeof(path), g->write_filename, (int) i);
        rc = raw ? ufoir_io_write_raw(path, vol + i * per, per) : ufoir_io_write_tiff(path, vol + i * per, n, n, 1);
        if (rc)
            ufoir__fail(ctx, rc, "write: %s", ufoir_io_last_error());
    }
    return rc;
}

int ufoir_graph_run(ufoir_ctx *ctx, const ufoir_graph *g, unsigned int *n_slices_out)
{
    if (!ctx || !g)
        return UFOIR_ERR_INVALID;
    if (n_slices_out)
        *n_slices_out = 0;
    if (g->read_path[0] == '\0' || g->write_filename[0] == '\0')
        return ufoir__fail(ctx, UFOIR_ERR_INVALID, "the graph needs a read node and a write node to run");
    float *sino = NULL, *vol = NULL;
    size_t S = 0;
    unsigned int w = 0, h = 0;
    ufoir_projector *proj = NULL;
    int rc = read_all(ctx, g, &sino, &S, &w, &h);
    if (rc)
        return rc;
    const size_t dims[2] = {w, h};           /* sinogram: dims[0] = n_dets, dims[1] = n_angles */
    vol = (float *) calloc((size_t) w * w * S, sizeof(float));
    if (!vol) {
        rc = ufoir__fail(ctx, UFOIR_ERR_NOMEM, "out of host memory");
        goto done;
    }
    if ((rc = ufoir_projector_create(ctx, &g->projector, &proj)))
        goto done;
    switch (g->method) {
    case UFOIR_METHOD_SART: rc = ufoir_sart_process(proj, &g->sart, sino, dims, vol, S); break;
    case UFOIR_METHOD_SIRT: rc = ufoir_sirt_process(proj, &g->sart, sino, dims, vol, S); break;
    case UFOIR_METHOD_ASDPOCS: rc = ufoir_asdpocs_process(proj, &g->asdpocs, sino, dims, vol, S); break;
    case UFOIR_METHOD_SBTV: rc = ufoir_sbtv_process(proj, &g->sbtv, sino, dims, vol, S); break;
    default: rc = ufoir__fail(ctx, UFOIR_ERR_INVALID, "graph without a method"); break;
    }
    if (rc)
        goto done;
    rc = write_all(ctx, g, vol, S, w);
    if (rc == UFOIR_OK && n_slices_out)
        *n_slices_out = (unsigned int) S;
done:
    ufoir_projector_destroy(proj);
    free(sino);
    free(vol);
    return rc;
}
