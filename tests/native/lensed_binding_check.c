/* Compiles the reference-side binding (include/lensed_gb300_lensed.h)
 * against Lensed's own headers and prior code (src/input.h, src/prior.h,
 * src/prior.c, the three prior kinds under src/prior/, src/parse.c, src/log.c, compiled where they
 * lie) and the library's C ABI: builds a Lensed `input` whose priors come
 * from the reference's prior_read(), turns it into the library's object
 * list and checks that the library composes and compiles the model
 * (lg_compile_check, no GPU needed).  Prints one line per prior string and
 * the check's status. */
#include <stdio.h>
#include <string.h>

#include "input.h"
#include "prior.h"
#include "lensed_gb300.h"
#include "lensed_gb300_lensed.h"

static void set(param* p, const char* name, const char* text, int wrap, int ipp)
{
    p->name = name;
    p->pri = text ? prior_read(text) : NULL;
    p->wrap = wrap;
    p->ipp = ipp;
}

int main(void)
{
    param lens[5], src[7], sky[3];
    object objs[3];
    input inp;
    lg_object_desc* od;
    lg_image_desc img;
    lg_options opt;
    char log[4096];
    size_t i, j;
    int rc;
    memset(lens, 0, sizeof lens);
    memset(src, 0, sizeof src);
    memset(sky, 0, sizeof sky);
    set(&lens[0], "x", "unif 20.25 28.125", 0, 0);
    set(&lens[1], "y", "norm 24.0 0.3", 0, 0);
    set(&lens[2], "r", "unif 5 12", 0, 0);
    set(&lens[3], "q", "unif 0.5 0.95", 0, 0);
    set(&lens[4], "pa", "unif 0 180", 1, 0); /* "wrap unif 0 180" in the ini */
    set(&src[0], "x", "unif 10 20", 0, 1);   /* "image unif 10 20" */
    set(&src[1], "y", "unif 25 35", 0, 1);
    set(&src[2], "r", "unif 1 3", 0, 0);
    set(&src[3], "mag", "unif -3 0", 0, 0);
    set(&src[4], "n", "norm 2.5 0.1234567890123", 0, 0);
    set(&src[5], "q", "unif 0.5 1", 0, 0);
    set(&src[6], "pa", "unif 0 180", 1, 0);
    set(&sky[0], "bg", "10.5", 0, 0);         /* a fixed value (delta prior) */
    set(&sky[1], "dx", NULL, 0, 0);            /* no prior: the plugin default */
    set(&sky[2], "dy", NULL, 0, 0);
    objs[0].name = "sie";
    objs[0].id = "lens";
    objs[0].npars = 5;
    objs[0].pars = lens;
    objs[1].name = "sersic";
    objs[1].id = "src";
    objs[1].npars = 7;
    objs[1].pars = src;
    objs[2].name = "sky";
    objs[2].id = "sky";
    objs[2].npars = 3;
    objs[2].pars = sky;
    inp.opts = NULL;
    inp.reqs = NULL;
    inp.nobjs = 3;
    inp.objs = objs;

    od = lensed_gb300_objects(&inp);
    if (!od) return 2;
    for (i = 0; i < inp.nobjs; ++i)
        for (j = 0; j < inp.objs[i].npars; ++j)
            printf("%s.%s = %s\n", od[i].id, inp.objs[i].pars[j].name, od[i].priors[j] ? od[i].priors[j] : "(default)");
    memset(&img, 0, sizeof img);
    img.width = 48;
    img.height = 40;
    opt.rule = "sub3";
    opt.device = 0;
    opt.max_batch = 16;
    opt.flags = 0;
    rc = lg_compile_check(&img, od, (int)inp.nobjs, &opt, log, sizeof log);
    printf("lg_compile_check %d %s\n", rc, rc ? log : "");
    lensed_gb300_free_objects(&inp, od);
    return rc == 0 ? 0 : 1;
}
