/* RSF file I/O for the drop-in programs (see rsfio.h). */
#define _GNU_SOURCE
#include "rsfio.h"

#include <ctype.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <unistd.h>

#define NAX 9

struct rsf_file {
    int output;
    FILE *hdr;              /* header stream (input: consumed; output: written at first write/close) */
    char hdr_path[4096];
    FILE *bin;              /* sample stream */
    char bin_path[4096];
    int inline_data;        /* samples follow the header in the same stream */
    int header_done;
    int n[NAX];
    float o[NAX], d[NAX];
    char label[NAX][32];
    int own_hdr;
    int cplx; /* native_complex samples */
};

static int g_argc;
static char **g_argv;
static char g_err[512];

static void set_err(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

const char *rsf_error(void) { return g_err; }

void rsf_init(int argc, char **argv) {
    g_argc = argc;
    g_argv = argv;
}

static const char *arg(const char *key) {
    size_t kl = strlen(key);
    const char *v = NULL;
    for (int i = 1; i < g_argc; i++)
        if (strncmp(g_argv[i], key, kl) == 0 && g_argv[i][kl] == '=') v = g_argv[i] + kl + 1;
    return v;
}

int rsf_get_int(const char *key, int *v) {
    const char *s = arg(key);
    if (!s) return 0;
    *v = atoi(s);
    return 1;
}

int rsf_get_float(const char *key, float *v) {
    const char *s = arg(key);
    if (!s) return 0;
    *v = (float)atof(s);
    return 1;
}

int rsf_get_bool(const char *key, int *v) {
    const char *s = arg(key);
    if (!s) return 0;
    *v = (s[0] == 'y' || s[0] == 'Y' || s[0] == '1' || s[0] == 't' || s[0] == 'T');
    return 1;
}

const char *rsf_get_string(const char *key) { return arg(key); }

/* parse key=value tokens (values may be double-quoted) from text */
static void parse(rsf_file *f, const char *text, char *in_path, size_t in_len, char *fmt, size_t fmt_len) {
    const char *p = text;
    while (*p) {
        while (*p && isspace((unsigned char)*p)) p++;
        const char *k = p;
        while (*p && *p != '=' && !isspace((unsigned char)*p)) p++;
        if (*p != '=') {
            while (*p && !isspace((unsigned char)*p)) p++;
            continue;
        }
        char key[64];
        size_t kl = (size_t)(p - k) < sizeof key - 1 ? (size_t)(p - k) : sizeof key - 1;
        memcpy(key, k, kl);
        key[kl] = 0;
        p++;
        char val[4096];
        size_t vl = 0;
        if (*p == '"') {
            p++;
            while (*p && *p != '"' && vl < sizeof val - 1) val[vl++] = *p++;
            if (*p == '"') p++;
        } else {
            while (*p && !isspace((unsigned char)*p) && vl < sizeof val - 1) val[vl++] = *p++;
        }
        val[vl] = 0;
        if (key[0] && (key[0] == 'n' || key[0] == 'o' || key[0] == 'd') && isdigit((unsigned char)key[1]) && !key[2]) {
            int a = key[1] - '1';
            if (a >= 0 && a < NAX) {
                if (key[0] == 'n') f->n[a] = atoi(val);
                else if (key[0] == 'o') f->o[a] = (float)atof(val);
                else f->d[a] = (float)atof(val);
            }
        } else if (strcmp(key, "in") == 0) {
            snprintf(in_path, in_len, "%s", val);
        } else if (strcmp(key, "data_format") == 0) {
            snprintf(fmt, fmt_len, "%s", val);
        }
    }
}

static rsf_file *new_file(void) {
    rsf_file *f = calloc(1, sizeof *f);
    for (int a = 0; a < NAX; a++) {
        f->n[a] = 1;
        f->d[a] = 1.f;
    }
    return f;
}

static rsf_file *open_input(const char *tag, const char *path) {
    rsf_file *f = new_file();
    FILE *h;
    if (!path && strcmp(tag, "in") == 0) {
        h = stdin;
        snprintf(f->hdr_path, sizeof f->hdr_path, "stdin");
    } else {
        if (!path) path = arg(tag);
        if (!path) {
            set_err("missing %s= argument", tag);
            free(f);
            return NULL;
        }
        snprintf(f->hdr_path, sizeof f->hdr_path, "%s", path);
        h = fopen(path, "rb");
        if (!h) {
            set_err("cannot open %s", path);
            free(f);
            return NULL;
        }
        f->own_hdr = 1;
    }
    /* header text up to EOF or the inline-data mark 0x0c 0x0c 0x04 */
    size_t cap = 1 << 16, len = 0;
    char *text = malloc(cap);
    int c, m1 = 0, m2 = 0;
    while ((c = fgetc(h)) != EOF) {
        if (m1 == 0x0c && m2 == 0x0c && c == 0x04) {
            len -= 2;
            f->inline_data = 1;
            break;
        }
        m1 = m2;
        m2 = c;
        if (len + 1 >= cap) text = realloc(text, cap *= 2);
        text[len++] = (char)c;
    }
    text[len] = 0;
    char in_path[4096] = "", fmt[64] = "native_float";
    parse(f, text, in_path, sizeof in_path, fmt, sizeof fmt);
    free(text);
    f->cplx = strcmp(fmt, "native_complex") == 0;
    if (strcmp(fmt, "native_float") != 0 && !f->cplx) {
        set_err("%s: only data_format=native_float or native_complex is supported (got %s)", f->hdr_path, fmt);
        free(f);
        return NULL;
    }
    if (f->inline_data) {
        f->bin = h;
    } else {
        if (f->own_hdr) fclose(h);
        if (!in_path[0]) {
            set_err("%s: header has no in=", f->hdr_path);
            free(f);
            return NULL;
        }
        snprintf(f->bin_path, sizeof f->bin_path, "%s", in_path);
        f->bin = fopen(in_path, "rb");
        if (!f->bin) {
            set_err("%s: cannot open samples %s", f->hdr_path, in_path);
            free(f);
            return NULL;
        }
    }
    return f;
}

rsf_file *rsf_input(const char *tag) { return open_input(tag, NULL); }
rsf_file *rsf_input_path(const char *path) { return open_input(path, path); }
int rsf_is_complex(const rsf_file *f) { return f->cplx; }
void rsf_set_complex(rsf_file *f, int on) { f->cplx = on != 0; }

rsf_file *rsf_output(const char *tag) {
    rsf_file *f = new_file();
    f->output = 1;
    if (strcmp(tag, "out") == 0) {
        f->hdr = stdout;
        struct stat st;
        char path[4096];
        ssize_t l = readlink("/proc/self/fd/1", path, sizeof path - 1);
        if (fstat(1, &st) == 0 && S_ISREG(st.st_mode) && l > 0) {
            path[l] = 0;
            snprintf(f->hdr_path, sizeof f->hdr_path, "%s", path);
            snprintf(f->bin_path, sizeof f->bin_path, "%s@", path);
        } else {
            f->inline_data = 1; /* pipe: samples follow the header */
            snprintf(f->hdr_path, sizeof f->hdr_path, "stdout");
        }
    } else {
        const char *path = arg(tag);
        if (!path) {
            set_err("missing %s= argument", tag);
            free(f);
            return NULL;
        }
        snprintf(f->hdr_path, sizeof f->hdr_path, "%s", path);
        snprintf(f->bin_path, sizeof f->bin_path, "%s@", path);
        f->hdr = fopen(path, "w");
        if (!f->hdr) {
            set_err("cannot create %s", path);
            free(f);
            return NULL;
        }
        f->own_hdr = 1;
    }
    return f;
}

int rsf_n(const rsf_file *f, int axis) { return (axis >= 1 && axis <= NAX) ? f->n[axis - 1] : 1; }
float rsf_o(const rsf_file *f, int axis) { return (axis >= 1 && axis <= NAX) ? f->o[axis - 1] : 0.f; }
float rsf_d(const rsf_file *f, int axis) { return (axis >= 1 && axis <= NAX) ? f->d[axis - 1] : 1.f; }

size_t rsf_size(const rsf_file *f) {
    size_t s = 1;
    for (int a = 0; a < NAX; a++) s *= (size_t)(f->n[a] > 0 ? f->n[a] : 1);
    return s;
}

void rsf_set_axis(rsf_file *f, int axis, int n, float o, float d, const char *label) {
    if (axis < 1 || axis > NAX) return;
    f->n[axis - 1] = n;
    f->o[axis - 1] = o;
    f->d[axis - 1] = d;
    snprintf(f->label[axis - 1], sizeof f->label[0], "%s", label ? label : "");
}

static int write_header(rsf_file *f) {
    if (f->header_done) return 0;
    FILE *h = f->hdr;
    int last = 0;
    for (int a = 0; a < NAX; a++)
        if (f->n[a] != 1) last = a;
    for (int a = 0; a <= last; a++) {
        fprintf(h, "n%d=%d o%d=%.9g d%d=%.9g", a + 1, f->n[a], a + 1, f->o[a], a + 1, f->d[a]);
        if (f->label[a][0]) fprintf(h, " label%d=\"%s\"", a + 1, f->label[a]);
        fputc('\n', h);
    }
    if (f->cplx) fprintf(h, "data_format=\"native_complex\" esize=8\n");
    else fprintf(h, "data_format=\"native_float\" esize=4\n");
    if (f->inline_data) {
        fprintf(h, "in=\"stdin\"\n");
        fputc(0x0c, h);
        fputc(0x0c, h);
        fputc(0x04, h);
        f->bin = h;
    } else {
        fprintf(h, "in=\"%s\"\n", f->bin_path);
        f->bin = fopen(f->bin_path, "wb");
        if (!f->bin) {
            set_err("cannot create %s", f->bin_path);
            return -1;
        }
    }
    fflush(h);
    f->header_done = 1;
    return 0;
}

size_t rsf_read(rsf_file *f, float *buf, size_t n) { return fread(buf, sizeof(float), n, f->bin); }

size_t rsf_write(rsf_file *f, const float *buf, size_t n) {
    if (write_header(f) != 0) return 0;
    return fwrite(buf, sizeof(float), n, f->bin);
}

int rsf_close(rsf_file *f) {
    if (!f) return 0;
    int rc = 0;
    if (f->output) {
        rc = write_header(f);
        if (f->bin && f->bin != f->hdr) fclose(f->bin);
        if (f->own_hdr) fclose(f->hdr);
        else fflush(f->hdr);
    } else {
        if (f->bin && f->bin != stdin) fclose(f->bin);
    }
    free(f);
    return rc;
}
