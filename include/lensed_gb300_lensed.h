/*
 * lensed_gb300_lensed.h -- reference-side binding: helpers for Lensed's C
 * host to describe its parsed input to liblensed_gb300.
 *
 * Include after Lensed's own "input.h" and "prior.h" (src/input.h,
 * src/prior.h) and "lensed_gb300.h".  Header-only (static functions), so it
 * adds no symbol to either program.  Everything it reads is public in the
 * reference: the object list of `input` (src/input.h:112-143), the fields of
 * `param` (src/input.h:76-110: id, wrap, ipp, pri) and the opaque prior's
 * accessors (src/prior.h: prior_pseudo, prior_apply, prior_lower,
 * prior_upper, prior_print).
 *
 * Lensed keeps a parameter's prior as an opaque `prior*` built from the ini
 * text by set_param_prior() (src/input/objects.c:329-358), which strips the
 * "wrap" and "image" keywords into param.wrap and param.ipp.  The library
 * takes priors as that ini text, so lensed_gb300_prior_text() rebuilds it:
 *   delta  (prior_pseudo)  "<value>"        value = prior_apply(pri, 0.5), exact
 *   unif   (prints "U(")   "unif <a> <b>"   a, b = prior_lower / prior_upper, exact
 *   norm   (prints "N(")   "norm <m> <s>"   m = (l + u) / 2, s = (u - l) / 14 from
 *                                           prior_lower / prior_upper = m -+ 7 s
 *                                           (src/prior/norm.c), within an ulp
 * with "wrap " and "image " in front as the flags say.  Numbers are written
 * with 17 significant digits (prior_print's "%g" keeps only 6).
 */
#ifndef LENSED_GB300_LENSED_H
#define LENSED_GB300_LENSED_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* The ini text of a parameter's prior, or "" when it has none (the plugin
 * default applies).  Returns 0, or -1 if buf (n bytes) is too small or the
 * prior's kind is unknown. */
static int lensed_gb300_prior_text(const param* par, char* buf, size_t n)
{
    char kind[8] = "";
    char num[96];
    size_t len = 0;
    int w;
    if (n == 0) return -1;
    buf[0] = '\0';
    if (!par->pri) return 0;
    if (par->wrap) len += (size_t)snprintf(buf + len, len < n ? n - len : 0, "wrap ");
    if (par->ipp) len += (size_t)snprintf(buf + len, len < n ? n - len : 0, "image ");
    if (prior_pseudo(par->pri)) {
        w = snprintf(num, sizeof num, "%.17g", prior_apply(par->pri, 0.5));
    } else {
        const double lo = prior_lower(par->pri), hi = prior_upper(par->pri);
        prior_print(par->pri, kind, sizeof kind); /* "U(..." or "N(...", cut to fit */
        if (kind[0] == 'U')
            w = snprintf(num, sizeof num, "unif %.17g %.17g", lo, hi);
        else if (kind[0] == 'N')
            w = snprintf(num, sizeof num, "norm %.17g %.17g", 0.5 * (lo + hi), (hi - lo) / 14.0);
        else
            return -1;
    }
    if (w < 0 || (size_t)w >= sizeof num) return -1;
    len += (size_t)snprintf(buf + len, len < n ? n - len : 0, "%s", num);
    return len < n ? 0 : -1;
}

/* The library's object list for Lensed's input: objs[i] = {name, id,
 * priors}, with the prior strings of lensed_gb300_prior_text().  The arrays
 * are allocated here; release them with lensed_gb300_free_objects().
 * Returns NULL on failure. */
static lg_object_desc* lensed_gb300_objects(const input* inp)
{
    size_t i, j;
    lg_object_desc* od = (lg_object_desc*)calloc(inp->nobjs ? inp->nobjs : 1, sizeof *od);
    if (!od) return NULL;
    for (i = 0; i < inp->nobjs; ++i) {
        const object* obj = &inp->objs[i];
        const char** pri = (const char**)calloc(obj->npars ? obj->npars : 1, sizeof *pri);
        od[i].name = obj->name;
        od[i].id = obj->id;
        od[i].priors = pri;
        if (!pri) goto fail;
        for (j = 0; j < obj->npars; ++j) {
            char buf[256];
            char* s;
            if (lensed_gb300_prior_text(&obj->pars[j], buf, sizeof buf)) goto fail;
            if (!buf[0]) continue; /* NULL: the plugin default */
            s = (char*)malloc(strlen(buf) + 1);
            if (!s) goto fail;
            strcpy(s, buf);
            pri[j] = s;
        }
    }
    return od;
fail:
    for (i = 0; i < inp->nobjs; ++i) {
        if (!od[i].priors) continue;
        for (j = 0; j < inp->objs[i].npars; ++j) free((char*)od[i].priors[j]);
        free((void*)od[i].priors);
    }
    free(od);
    return NULL;
}

static void lensed_gb300_free_objects(const input* inp, lg_object_desc* od)
{
    size_t i, j;
    if (!od) return;
    for (i = 0; i < inp->nobjs; ++i) {
        for (j = 0; j < inp->objs[i].npars; ++j) free((char*)od[i].priors[j]);
        free((void*)od[i].priors);
    }
    free(od);
}

#endif
