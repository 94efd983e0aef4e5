/* Driver around the reference's own program generator (src/kernel.c) --
 * TEST INFRASTRUCTURE ONLY (see oracle/build_ref.py).
 *
 *   ref_gen meta <object>
 *       prints object_program(<object>): the reference's introspection
 *       program (kernel/object.cl, kernel/constants.cl, the object file and
 *       the generated meta_/params_ kernels)
 *   ref_gen main <W> <H> <psf> <psfw> <psfh> <nq> <nobjs> {<name> <type> <size> <types> <ipp>}...
 *       prints the -D options of kernel_options() as #define lines, then
 *       main_program(): plugins, generated compute() and set_params, and
 *       kernel/lensed.cl.  <type> is L/S/F, <size> the data size in floats,
 *       <types> the comma-separated parameter types, <ipp> 1 if the object's
 *       (x, y) pair has an image-plane prior.
 *
 * Linked with the reference's src/kernel.c, compiled from its own tree. */
#include <limits.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "input.h"
#include "kernel.h"

const char* LENSED_PATH = NULL;

/* The generator's second pass calls snprintf with a bound of (size_t)-1 to
 * mean "unbounded" (src/kernel.c:446 with :459-651); current glibc computes
 * the end of the buffer from that bound, overflows the pointer and writes
 * nothing.  This definition takes precedence over the C library's for the
 * generator and clamps the bound to INT_MAX, which is what the code
 * assumes. */
int snprintf(char* s, size_t n, const char* fmt, ...)
{
    va_list a;
    va_start(a, fmt);
    if (n > INT_MAX) n = INT_MAX;
    int r = vsnprintf(s, n, fmt, a);
    va_end(a);
    return r;
}

void verbose(const char* msg, ...) { (void)msg; }
void error(const char* msg, ...)
{
    va_list a;
    va_start(a, msg);
    vfprintf(stderr, msg, a);
    va_end(a);
    fputc('\n', stderr);
    exit(2);
}
void errori(const char* msg, ...)
{
    (void)msg;
    fputs("internal error\n", stderr);
    exit(2);
}

static void print_program(size_t n, const char** k)
{
    for (size_t i = 0; i < n; ++i) fputs(k[i], stdout);
}

int main(int argc, char** argv)
{
    const char* root = getenv("LENSED_SOURCE");
    if (!root || argc < 3) {
        fputs("usage: LENSED_SOURCE=<tree>/ ref_gen meta <object> | main ...\n", stderr);
        return 1;
    }
    LENSED_PATH = root;
    size_t n;
    const char** k;
    if (strcmp(argv[1], "meta") == 0) {
        object_program(argv[2], &n, &k);
        print_program(n, k);
        return 0;
    }
    if (strcmp(argv[1], "main") != 0 || argc < 9) return 1;
    size_t W = strtoul(argv[2], 0, 10), H = strtoul(argv[3], 0, 10);
    int psf = atoi(argv[4]);
    size_t pw = strtoul(argv[5], 0, 10), ph = strtoul(argv[6], 0, 10), nq = strtoul(argv[7], 0, 10);
    size_t nobjs = strtoul(argv[8], 0, 10);
    if ((size_t)argc != 9 + 5 * nobjs) return 1;
    object* objs = calloc(nobjs, sizeof(object));
    for (size_t i = 0; i < nobjs; ++i) {
        char** a = argv + 9 + 5 * i;
        objs[i].name = a[0];
        objs[i].id = a[0];
        objs[i].type = a[1][0];
        objs[i].size = strtoul(a[2], 0, 10);
        size_t np = 1;
        for (const char* c = a[3]; *c; ++c)
            if (*c == ',') ++np;
        objs[i].npars = np;
        objs[i].pars = calloc(np, sizeof(param));
        const char* c = a[3];
        int ipp = atoi(a[4]);
        for (size_t j = 0; j < np; ++j) {
            objs[i].pars[j].type = (int)strtol(c, (char**)&c, 10);
            if (*c == ',') ++c;
            objs[i].pars[j].ipp = ipp && (objs[i].pars[j].type == PAR_POSITION_X ||
                                          objs[i].pars[j].type == PAR_POSITION_Y);
        }
    }
    const char* flags[] = {NULL};
    const char* opts = kernel_options(W, H, psf, pw, ph, nq, flags);
    /* " -DNAME=value ..." -> #define lines */
    char* o = strdup(opts);
    for (char* t = strtok(o, " "); t; t = strtok(NULL, " ")) {
        if (strncmp(t, "-D", 2) != 0) continue;
        char* eq = strchr(t, '=');
        if (eq) {
            *eq = ' ';
        }
        printf("#define %s\n", t + 2);
    }
    fputs("//@@program@@\n", stdout);
    main_program(nobjs, objs, &n, &k);
    print_program(n, k);
    return 0;
}
