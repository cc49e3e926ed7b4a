/* Implementation of the minimal RSF stand-in declared in rsf.h.
 *
 * Files: an RSF header is a text file of key=value pairs; the samples live in
 * a separate binary file named by the header's in="..." entry
 * (data_format=native_float, esize=4, or native_complex, esize=8).  Output headers are written at the
 * first sample write and rewritten at exit, so axes set late are kept.
 * The tags "in" and "out" are standard input and output; for "out" the binary
 * file is <path of stdout>@.  Any other tag names a file on the command line
 * (tag=path); an input tag with no such parameter is itself the file name
 * (as sf_input treats it).  Outputs start with the keys of the standard
 * input's header, as Madagascar's do.
 *
 * Test infrastructure for the oracle's checker; not product code. */
#define _GNU_SOURCE
#include "rsf.h"

#include <stdarg.h>
#include <unistd.h>

#define MAXKEYS 64

struct sf_Axis {
    int n;
    float o, d;
    char label[64];
    char unit[64];
};

struct sf_File {
    int output;
    char hdr_path[4096];
    char bin_path[4096];
    FILE *bin;
    int nkeys;
    char keys[MAXKEYS][32];
    char vals[MAXKEYS][256];
    int header_written;
    sf_datatype type;
};

static int g_argc = 0;
static char **g_argv = NULL;
static struct sf_File *g_outputs[16];
static struct sf_File *g_in = NULL; /* standard input, whose header outputs inherit */
static int g_nout = 0;

static const char *arg_value(const char *key) {
    size_t kl = strlen(key);
    const char *found = NULL;
    for (int i = 1; i < g_argc; i++) {
        if (strncmp(g_argv[i], key, kl) == 0 && g_argv[i][kl] == '=') found = g_argv[i] + kl + 1;
    }
    return found;
}

static void write_header(struct sf_File *f) {
    FILE *h = fopen(f->hdr_path, "w");
    if (!h) sf_error("cannot write header %s", f->hdr_path);
    for (int i = 0; i < f->nkeys; i++) fprintf(h, "%s=%s\n", f->keys[i], f->vals[i]);
    if (f->type == SF_COMPLEX) fprintf(h, "data_format=\"native_complex\"\nesize=8\nin=\"%s\"\n", f->bin_path);
    else fprintf(h, "data_format=\"native_float\"\nesize=4\nin=\"%s\"\n", f->bin_path);
    fclose(h);
    f->header_written = 1;
}

static void flush_outputs(void) {
    for (int i = 0; i < g_nout; i++) {
        if (g_outputs[i]->bin) fflush(g_outputs[i]->bin);
        write_header(g_outputs[i]);
    }
}

void sf_init(int argc, char **argv) {
    g_argc = argc;
    g_argv = argv;
    atexit(flush_outputs);
}

char *sf_getstring(const char *key) {
    const char *v = arg_value(key);
    if (!v) return NULL;
    char *s = strdup(v);
    size_t l = strlen(s);
    if (l >= 2 && s[0] == '"' && s[l - 1] == '"') {
        memmove(s, s + 1, l - 2);
        s[l - 2] = 0;
    }
    return s;
}

bool sf_getbool(const char *key, bool *par) {
    const char *v = arg_value(key);
    if (!v) return false;
    *par = (v[0] == 'y' || v[0] == 'Y' || v[0] == '1' || v[0] == 't' || v[0] == 'T');
    return true;
}

bool sf_getint(const char *key, int *par) {
    const char *v = arg_value(key);
    if (!v) return false;
    *par = atoi(v);
    return true;
}

bool sf_getfloat(const char *key, float *par) {
    const char *v = arg_value(key);
    if (!v) return false;
    *par = (float)atof(v);
    return true;
}

static void set_key(struct sf_File *f, const char *k, const char *v) {
    for (int i = 0; i < f->nkeys; i++) {
        if (strcmp(f->keys[i], k) == 0) {
            snprintf(f->vals[i], sizeof f->vals[i], "%s", v);
            return;
        }
    }
    if (f->nkeys >= MAXKEYS) sf_error("too many header keys");
    snprintf(f->keys[f->nkeys], sizeof f->keys[0], "%s", k);
    snprintf(f->vals[f->nkeys], sizeof f->vals[0], "%s", v);
    f->nkeys++;
}

static const char *get_key(struct sf_File *f, const char *k) {
    for (int i = 0; i < f->nkeys; i++)
        if (strcmp(f->keys[i], k) == 0) return f->vals[i];
    return NULL;
}

static void parse_header(struct sf_File *f, FILE *h) {
    char tok[512];
    while (fscanf(h, "%511s", tok) == 1) {
        char *eq = strchr(tok, '=');
        if (!eq) continue;
        *eq = 0;
        char *v = eq + 1;
        size_t l = strlen(v);
        if (l >= 2 && v[0] == '"' && v[l - 1] == '"') {
            v[l - 1] = 0;
            v++;
        }
        set_key(f, tok, v);
    }
}

sf_file sf_input(const char *tag) {
    struct sf_File *f = calloc(1, sizeof *f);
    FILE *h;
    if (strcmp(tag, "in") == 0) {
        h = stdin;
        snprintf(f->hdr_path, sizeof f->hdr_path, "stdin");
    } else {
        const char *p = arg_value(tag);
        if (!p) p = tag; /* a file name given as such */
        snprintf(f->hdr_path, sizeof f->hdr_path, "%s", p);
        h = fopen(p, "r");
        if (!h) sf_error("cannot open %s", p);
    }
    parse_header(f, h);
    if (h != stdin) fclose(h);
    const char *fmt = get_key(f, "data_format");
    f->type = (fmt && strstr(fmt, "complex")) ? SF_COMPLEX : SF_FLOAT;
    if (strcmp(tag, "in") == 0) g_in = f;
    const char *in = get_key(f, "in");
    if (!in) sf_error("header %s has no in=", f->hdr_path);
    snprintf(f->bin_path, sizeof f->bin_path, "%s", in);
    f->bin = fopen(f->bin_path, "rb");
    if (!f->bin) sf_error("cannot open binary %s", f->bin_path);
    return f;
}

sf_file sf_output(const char *tag) {
    struct sf_File *f = calloc(1, sizeof *f);
    f->output = 1;
    f->type = SF_FLOAT;
    if (g_in) { /* an output starts as a copy of the standard input's header */
        for (int i = 0; i < g_in->nkeys; i++)
            if (strcmp(g_in->keys[i], "in") && strcmp(g_in->keys[i], "data_format") && strcmp(g_in->keys[i], "esize"))
                set_key(f, g_in->keys[i], g_in->vals[i]);
        f->type = g_in->type;
    }
    if (strcmp(tag, "out") == 0) {
        ssize_t l = readlink("/proc/self/fd/1", f->hdr_path, sizeof f->hdr_path - 1);
        if (l <= 0) sf_error("cannot resolve stdout path");
        f->hdr_path[l] = 0;
    } else {
        const char *p = arg_value(tag);
        if (!p) sf_error("missing %s= argument", tag);
        snprintf(f->hdr_path, sizeof f->hdr_path, "%s", p);
    }
    snprintf(f->bin_path, sizeof f->bin_path, "%s@", f->hdr_path);
    if (g_nout < 16) g_outputs[g_nout++] = f;
    return f;
}

sf_axis sf_maxa(int n, float o, float d) {
    struct sf_Axis *a = calloc(1, sizeof *a);
    a->n = n;
    a->o = o;
    a->d = d;
    return a;
}

sf_axis sf_iaxa(sf_file f, int i) {
    char k[16];
    const char *v;
    struct sf_Axis *a = calloc(1, sizeof *a);
    snprintf(k, sizeof k, "n%d", i);
    v = get_key(f, k);
    a->n = v ? atoi(v) : 1;
    snprintf(k, sizeof k, "o%d", i);
    v = get_key(f, k);
    a->o = v ? (float)atof(v) : 0.f;
    snprintf(k, sizeof k, "d%d", i);
    v = get_key(f, k);
    a->d = v ? (float)atof(v) : 1.f;
    return a;
}

void sf_oaxa(sf_file f, sf_axis a, int i) {
    char k[16], v[64];
    snprintf(k, sizeof k, "n%d", i);
    snprintf(v, sizeof v, "%d", a->n);
    set_key(f, k, v);
    snprintf(k, sizeof k, "o%d", i);
    snprintf(v, sizeof v, "%.9g", a->o);
    set_key(f, k, v);
    snprintf(k, sizeof k, "d%d", i);
    snprintf(v, sizeof v, "%.9g", a->d);
    set_key(f, k, v);
}

void sf_raxa(sf_axis a) { fprintf(stderr, "n=%d o=%g d=%g %s\n", a->n, a->o, a->d, a->label); }
int sf_n(sf_axis a) { return a->n; }
float sf_o(sf_axis a) { return a->o; }
float sf_d(sf_axis a) { return a->d; }
void sf_setn(sf_axis a, int n) { a->n = n; }
void sf_seto(sf_axis a, float o) { a->o = o; }
void sf_setd(sf_axis a, float d) { a->d = d; }
void sf_setlabel(sf_axis a, const char *label) { snprintf(a->label, sizeof a->label, "%s", label); }
void sf_setunit(sf_axis a, const char *unit) { snprintf(a->unit, sizeof a->unit, "%s", unit); }

void sf_floatread(float *arr, size_t n, sf_file f) {
    if (fread(arr, sizeof(float), n, f->bin) != n) sf_error("short read from %s", f->bin_path);
}

void sf_floatwrite(float *arr, size_t n, sf_file f) {
    if (!f->bin) {
        f->bin = fopen(f->bin_path, "wb");
        if (!f->bin) sf_error("cannot open %s", f->bin_path);
        write_header(f);
    }
    if (fwrite(arr, sizeof(float), n, f->bin) != n) sf_error("short write to %s", f->bin_path);
}

void sf_settype(sf_file f, sf_datatype t) { f->type = t; }
sf_datatype sf_gettype(sf_file f) { return f->type; }

void sf_fileclose(sf_file f) {
    if (!f->output && f->bin) { /* outputs keep their stream: headers are rewritten at exit */
        fclose(f->bin);
        f->bin = NULL;
    }
}

sf_complex *sf_complexalloc(size_t n) { return (sf_complex *)sf_alloc(n, sizeof(sf_complex)); }
bool *sf_boolalloc(size_t n) { return (bool *)sf_alloc(n, sizeof(bool)); }
off_t *sf_largeintalloc(size_t n) { return (off_t *)sf_alloc(n, sizeof(off_t)); }

void sf_complexread(sf_complex *arr, size_t n, sf_file f) {
    if (fread(arr, sizeof(sf_complex), n, f->bin) != n) sf_error("short read from %s", f->bin_path);
}

void sf_complexwrite(sf_complex *arr, size_t n, sf_file f) {
    if (!f->bin) {
        f->bin = fopen(f->bin_path, "wb");
        if (!f->bin) sf_error("cannot open %s", f->bin_path);
        write_header(f);
    }
    if (fwrite(arr, sizeof(sf_complex), n, f->bin) != n) sf_error("short write to %s", f->bin_path);
}

void sf_seek(sf_file f, off_t offset, int whence) {
    if (fseeko(f->bin, offset, whence) != 0) sf_error("seek failed on %s", f->bin_path);
}

void *sf_alloc(size_t n, size_t size) {
    void *p = malloc(n * size ? n * size : 1);
    if (!p) sf_error("out of memory");
    return p;
}
float *sf_floatalloc(size_t n) { return (float *)sf_alloc(n, sizeof(float)); }
int *sf_intalloc(size_t n) { return (int *)sf_alloc(n, sizeof(int)); }

float **sf_floatalloc2(size_t n1, size_t n2) {
    float **p = (float **)sf_alloc(n2, sizeof(float *));
    p[0] = sf_floatalloc(n1 * n2);
    for (size_t i = 1; i < n2; i++) p[i] = p[0] + i * n1;
    return p;
}

int **sf_intalloc2(size_t n1, size_t n2) {
    int **p = (int **)sf_alloc(n2, sizeof(int *));
    p[0] = sf_intalloc(n1 * n2);
    for (size_t i = 1; i < n2; i++) p[i] = p[0] + i * n1;
    return p;
}

float ***sf_floatalloc3(size_t n1, size_t n2, size_t n3) {
    float ***p = (float ***)sf_alloc(n3, sizeof(float **));
    p[0] = sf_floatalloc2(n1, n2 * n3);
    for (size_t i = 1; i < n3; i++) p[i] = p[0] + i * n2;
    return p;
}

void sf_warning(const char *format, ...) {
    va_list ap;
    va_start(ap, format);
    vfprintf(stderr, format, ap);
    va_end(ap);
    fputc('\n', stderr);
}

void sf_error(const char *format, ...) {
    va_list ap;
    va_start(ap, format);
    fprintf(stderr, "rsf-shim error: ");
    vfprintf(stderr, format, ap);
    va_end(ap);
    fputc('\n', stderr);
    exit(1);
}

void pt2dread1(sf_file F, pt2d *v, size_t n, int k) {
    float w[3];
    for (size_t i = 0; i < n; i++) {
        sf_floatread(w, (size_t)k, F);
        v[i].x = w[0];
        v[i].z = w[1];
        v[i].v = (k == 3) ? w[2] : 0.f;
    }
}

void pt3dread1(sf_file F, pt3d *v, size_t n, int k) {
    float w[4];
    for (size_t i = 0; i < n; i++) {
        sf_floatread(w, (size_t)k, F);
        v[i].x = w[0];
        v[i].y = w[1];
        v[i].z = w[2];
        v[i].v = (k == 4) ? w[3] : 0.f;
    }
}

pt2d *pt2dalloc1(size_t n) { return (pt2d *)sf_alloc(n, sizeof(pt2d)); }
pt3d *pt3dalloc1(size_t n) { return (pt3d *)sf_alloc(n, sizeof(pt3d)); }
void printpt2d(pt2d P) { fprintf(stderr, "P: x=%f z=%f v=%f\n", P.x, P.z, P.v); }
void printpt3d(pt3d P) { fprintf(stderr, "P: x=%f y=%f z=%f v=%f\n", P.x, P.y, P.z, P.v); }

/* libsu's 8-point sinc interpolator is reached only through the reference's
 * sinc=y option, which the oracle never uses; the stand-in refuses loudly. */
void ints8r(int nxin, float dxin, float fxin, float yin[], float yinl, float yinr, int nxout, float xout[],
            float yout[]) {
    (void)nxin; (void)dxin; (void)fxin; (void)yin; (void)yinl; (void)yinr; (void)nxout; (void)xout; (void)yout;
    sf_error("sinc interpolation (sinc=y) is not provided by the RSF stand-in");
}
