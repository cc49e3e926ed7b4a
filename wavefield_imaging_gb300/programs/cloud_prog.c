/* Drop-in replacements for the reference's point-cloud programs
 *   sfbycloudwin3d   (CODE/Mbycloudwin3d.c)
 *   sfbycloudmerge3d (CODE/Mbycloudmerge3d.c with CODE/hash.c)
 * on the engine's C-ABI (awe_cloud_window, awe_cloud_merge).  Usage as the
 * reference:
 *
 *   sfbycloudwin3d < cloud.rsf oo=orbit.rsf dat=data.rsf dout=wdata.rsf [apt=15] > wcloud.rsf
 *   sfbycloudmerge3d wcloud1.rsf ... wcloudN.rsf wdata1.rsf ... wdataN.rsf all=cloud.rsf [norm=y] > data.rsf
 *
 * Window: cloud points n1=9 (x, y, z, normal, 3 more) by n2 points, orbit
 * the same layout (x, y, z used), complex data [nf][ng]; the kept points go
 * to standard output (n1=9, n2=nw) and their data columns to dout
 * (complex, n1=nw, n2=nf).  fast=n (the reference's out-of-core pass)
 * writes the same points and no data.  With no point kept the outputs hold
 * n2=0 (the reference writes one zero point and unset data then).
 * Merge: the first half of the file arguments are the windows' clouds, the
 * second half their data (float or complex); all= the full cloud; the sum
 * over windows [nf][na] goes to standard output, divided by the fold with
 * norm=y; hashscale= (default 2) sizes the lookup table.
 * gpu= selects the device (default 0).  Errors print to stderr and exit 1. */
#include <libgen.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "awe.h"
#include "rsfio.h"

static void die(const char *what, const char *msg) {
    fprintf(stderr, "%s: %s\n", what, msg);
    exit(1);
}

static float *read_all(rsf_file *f, size_t n, const char *prog, const char *what) {
    float *b = malloc(sizeof(float) * (n ? n : 1));
    if (rsf_read(f, b, n) != n) die(prog, what);
    return b;
}

static int window_main(const char *prog, int gpu) {
    float apt = 15.f;
    int fast = 1;
    rsf_get_float("apt", &apt);
    rsf_get_bool("fast", &fast);
    rsf_file *Fin = rsf_input("in"), *Fo = rsf_input("oo"), *Fdat = rsf_input("dat");
    if (!Fin || !Fo || !Fdat) die(prog, rsf_error());
    if (rsf_n(Fin, 1) != AWE_CLOUD_NCO || rsf_n(Fo, 1) != AWE_CLOUD_NCO) die(prog, "clouds need n1=9");
    if (!rsf_is_complex(Fdat)) die(prog, "dat= must be complex (data_format=native_complex)");
    const long long ng = rsf_n(Fin, 2), no = rsf_n(Fo, 2), nf = rsf_n(Fdat, 2);
    if (rsf_n(Fdat, 1) != ng) die(prog, "dat= n1 must equal the number of ground points");
    float *g = read_all(Fin, (size_t)ng * AWE_CLOUD_NCO, prog, "short read (cloud)");
    float *o = read_all(Fo, (size_t)no * AWE_CLOUD_NCO, prog, "short read (orbit)");
    float *d = fast ? read_all(Fdat, (size_t)nf * ng * 2, prog, "short read (dat)") : NULL;
    long long nw = 0;
    long long *index = malloc(sizeof(long long) * (ng ? ng : 1));
    float *win = malloc(sizeof(float) * AWE_CLOUD_NCO * (ng ? ng : 1));
    float *wd = fast ? malloc(sizeof(float) * 2 * (nf * ng > 0 ? nf * ng : 1)) : NULL;
    if (awe_cloud_window(gpu, g, ng, o, no, apt, fast ? nf : 0, 2, d, &nw, index, win, wd) != AWE_OK)
        die(prog, awe_last_error());
    rsf_file *Fgou = rsf_output("out");
    if (!Fgou) die(prog, rsf_error());
    rsf_set_axis(Fgou, 1, AWE_CLOUD_NCO, rsf_o(Fin, 1), rsf_d(Fin, 1), "");
    rsf_set_axis(Fgou, 2, (int)nw, 0.f, 1.f, "");
    if (rsf_write(Fgou, win, (size_t)nw * AWE_CLOUD_NCO) != (size_t)nw * AWE_CLOUD_NCO && nw > 0)
        die(prog, "short write (window cloud)");
    rsf_close(Fgou);
    if (fast) {
        rsf_file *Fdou = rsf_output("dout");
        if (!Fdou) die(prog, rsf_error());
        rsf_set_complex(Fdou, 1);
        rsf_set_axis(Fdou, 1, (int)nw, 0.f, 1.f, "");
        rsf_set_axis(Fdou, 2, (int)nf, rsf_o(Fdat, 2), rsf_d(Fdat, 2), "t");
        if (rsf_write(Fdou, wd, (size_t)nf * nw * 2) != (size_t)nf * nw * 2 && nf * nw > 0)
            die(prog, "short write (window data)");
        rsf_close(Fdou);
    }
    rsf_close(Fin);
    rsf_close(Fo);
    rsf_close(Fdat);
    free(g);
    free(o);
    free(d);
    free(index);
    free(win);
    free(wd);
    return 0;
}

static int merge_main(const char *prog, int gpu, int argc, char **argv) {
    int norm = 1;
    float hashscale = 2.f;
    rsf_get_bool("norm", &norm);
    rsf_get_float("hashscale", &hashscale);
    /* file arguments: every argument without '=' (Mbycloudmerge3d.c:70-83) */
    const char **names = malloc(sizeof(char *) * (size_t)argc);
    int nfiles = 0;
    for (int i = 1; i < argc; i++)
        if (!strchr(argv[i], '=')) names[nfiles++] = argv[i];
    if (nfiles == 0) die(prog, "no input");
    const int nwin = nfiles / 2;
    rsf_file *Fall = rsf_input("all");
    if (!Fall) die(prog, rsf_error());
    if (rsf_n(Fall, 1) != AWE_CLOUD_NCO) die(prog, "all= needs n1=9");
    const long long na = rsf_n(Fall, 2);
    float *all = read_all(Fall, (size_t)na * AWE_CLOUD_NCO, prog, "short read (all)");
    long long *nwp = malloc(sizeof(long long) * (nwin ? nwin : 1));
    long long ntot = 0, nf = 0;
    int ncomp = 1;
    float of = 0.f, df = 1.f;
    /* sizes first, then one pass reading every window's points and data */
    for (int c = 0; c < nwin; c++) {
        rsf_file *Fc = rsf_input_path(names[c]), *Fd = rsf_input_path(names[c + nwin]);
        if (!Fc || !Fd) die(prog, rsf_error());
        nwp[c] = rsf_n(Fc, 2);
        if (nwp[c] > 0 && rsf_n(Fc, 1) != AWE_CLOUD_NCO) die(prog, "window clouds need n1=9");
        if (c == 0) {
            nf = rsf_n(Fd, 2);
            ncomp = rsf_is_complex(Fd) ? 2 : 1;
            of = rsf_o(Fd, 2);
            df = rsf_d(Fd, 2);
        }
        ntot += nwp[c];
        rsf_close(Fc);
        rsf_close(Fd);
    }
    float *pts = malloc(sizeof(float) * AWE_CLOUD_NCO * (ntot ? ntot : 1));
    float *dat = malloc(sizeof(float) * (size_t)ncomp * (ntot * nf > 0 ? ntot * nf : 1));
    long long p0 = 0;
    for (int c = 0; c < nwin; c++) {
        if (nwp[c] == 0) continue; /* empty windows are skipped (Mbycloudmerge3d.c:199) */
        rsf_file *Fc = rsf_input_path(names[c]), *Fd = rsf_input_path(names[c + nwin]);
        if (!Fc || !Fd) die(prog, rsf_error());
        if ((rsf_is_complex(Fd) ? 2 : 1) != ncomp || rsf_n(Fd, 2) != nf || rsf_n(Fd, 1) != nwp[c])
            die(prog, "window data files differ in type or size");
        if (rsf_read(Fc, pts + p0 * AWE_CLOUD_NCO, (size_t)nwp[c] * AWE_CLOUD_NCO) != (size_t)nwp[c] * AWE_CLOUD_NCO)
            die(prog, "short read (window cloud)");
        if (rsf_read(Fd, dat + p0 * nf * ncomp, (size_t)nwp[c] * nf * ncomp) != (size_t)nwp[c] * nf * ncomp)
            die(prog, "short read (window data)");
        p0 += nwp[c];
        rsf_close(Fc);
        rsf_close(Fd);
    }
    float *out = malloc(sizeof(float) * (size_t)ncomp * (nf * na > 0 ? nf * na : 1));
    if (awe_cloud_merge(gpu, all, na, nwin, nwp, pts, dat, nf, ncomp, norm, hashscale, out) != AWE_OK)
        die(prog, awe_last_error());
    rsf_file *Fout = rsf_output("out");
    if (!Fout) die(prog, rsf_error());
    rsf_set_complex(Fout, ncomp == 2);
    rsf_set_axis(Fout, 1, (int)na, rsf_o(Fall, 2), rsf_d(Fall, 2), "");
    rsf_set_axis(Fout, 2, (int)nf, of, df, "");
    if (rsf_write(Fout, out, (size_t)nf * na * ncomp) != (size_t)nf * na * ncomp) die(prog, "short write");
    rsf_close(Fout);
    rsf_close(Fall);
    free(names);
    free(all);
    free(nwp);
    free(pts);
    free(dat);
    free(out);
    return 0;
}

int main(int argc, char **argv) {
    rsf_init(argc, argv);
    char name[256];
    snprintf(name, sizeof name, "%s", argv[0]);
    const char *prog = basename(name);
    int gpu = 0;
    rsf_get_int("gpu", &gpu);
    if (strstr(prog, "cloudwin3d")) return window_main(prog, gpu);
    if (strstr(prog, "cloudmerge3d")) return merge_main(prog, gpu, argc, argv);
    die(prog, "run as sfbycloudwin3d or sfbycloudmerge3d");
    return 1;
}
