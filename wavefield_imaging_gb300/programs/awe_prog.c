/* Drop-in replacements for the reference's RSF programs
 *   sfAWEFDcart2Dgpu  (CODE/MAWEFDcart2Dgpu.cu)
 *   sfAWEFDcart3Dgpu  (CODE/MAWEFDcart3Dgpu.cu)
 *   sfAWEFDspher2Dgpu (CODE/MAWEFDspher2Dgpu.cu)
 *   sfAWEFDspher3Dgpu (CODE/MAWEFDspher3Dgpu.cu)
 *   sfAWEFDcart2Dcpu  (CODE/MAWEFDcart2Dcpu.c, run on the GPU)
 *   sfAWEFDcart3Dcpu  (CODE/MAWEFDcart3Dcpu.c, run on the GPU)
 *   sfDYNAWEFDcart2Dgpu (CODE/MDYNAWEFDcart2Dgpu.cu: moving sources and
 *     receivers, sou/rec n2 = points per step, n3 = table rows)
 * on the engine's C-ABI (include/awe.h).  One source; the program name picks
 * the geometry and the scheme.  Usage as the reference:
 *
 *   sfAWEFDcart2Dgpu < wav.rsf vel=vel.rsf sou=sou.rsf rec=rec.rsf [rfl=rfl.rsf] wfl=wfl.rsf > dat.rsf [params]
 *
 * Parameters and defaults are those of each program's main() (cited below).
 * Extra parameter: precision=exact|fast (default fast; exact reproduces the
 * reference's float/double evaluation bit for bit).
 * adj=y (backward injection):
 *   sfAWEFDcart2Dcpu (MAWEFDcart2Dcpu.c:304-316, :353-369): expl=n injects
 *   the traces on standard input ([nt][nr]) at the receivers, expl=y the
 *   one-component wavelet at the sources, both reversed in time; the run
 *   stops after step nt-kt, whose wavefield (model window) is written to
 *   standard output as the image (axes z, x); no traces are written.
 *   kt=0 (the reference's default) never reaches the image step there and
 *   writes no image, so kt must be in [1, nt] here.
 *   sfAWEFDcart3Dcpu (MAWEFDcart3Dcpu.c:304-316): the wavelet reversed in
 *   time is injected at the sources; traces and snapshots as in a forward run.
 *   sfAWEFDspher3Dgpu (MAWEFDspher3Dgpu.cu:452-463, :533-563): the traces on
 *   standard input ([nt][nr]) go back in at the receivers, unscaled and
 *   reversed in time (inject_sources_3D_adj, spher_kernels.cu:367-398); no
 *   traces; snap=y writes the frames of the steps it % jsnap == 0 and of step
 *   nt-kt; after step nt-kt its model window is the image (axes ra, th, ph)
 *   on standard output.  kt in [1, nt] as above.
 * Snapshot windows of the cpu programs (snap=y; MAWEFDcart2Dcpu.c:186-205,
 * MAWEFDcart3Dcpu.c:180-203): nq*, oq*, dq* per axis, defaults the model's
 * axes; frames hold nq* samples from padded index floor((oq - opad)/d) with
 * stride floor(dq/d) (fdutil.c cut2d, cut3d_slice; opad = o - nb*d).  bnds=y
 * writes whole padded frames in 2D (the window then only sets the adj=y
 * image axes) and, in 3D, whole padded z-x planes of the nypad y planes the
 * y window picks (MAWEFDcart3Dcpu.c:341-353).  A window that leaves the
 * padded grid is an error (the reference reads outside its arrays); so is
 * adj=y with a window whose nqz, nqx differ from the model's (the image
 * buffer has the window's size, MAWEFDcart2Dcpu.c:247, :356-366).
 * Not provided: adj=y for sfAWEFDcart2Dgpu (its back-injection indexes the
 * source weight tables with receiver indices, MAWEFDcart2Dgpu.cu:391-394) and
 * the gpu programs that read no adj= (cart 3D, spher 2D) and sinc=y
 * injection (they stop with an error).
 * sfAWEFDcart3Dcpu bnds=y without oqy: the reference starts the y planes at
 * index nb of the padded grid and reads nb planes past its end; here the
 * nypad planes of the padded grid are written (the frames of oqy = oy - nb*dy).
 * Header differences: sfAWEFDspher3Dgpu's data and wavefield headers hold
 * the rows and frames actually written (the reference declares nt/jdata rows
 * and one frame more than it writes), and so does sfAWEFDcart2Dcpu adj=y
 * snap=y (the reference declares the frames of all nt steps).
 * Errors print to stderr and exit 1, as sf_error. */
#include <libgen.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "awe.h"
#include "rsfio.h"

static void die(const char *what, const char *msg) {
    fprintf(stderr, "%s: %s\n", what, msg);
    exit(1);
}

static rsf_file *g_wfl = NULL;

/* adj=y image runs (sfAWEFDcart2Dcpu, sfAWEFDspher3Dgpu): the image is the
 * frame of step img_it, cut from the padded frame when bnds=y; snapshot
 * frames go to wfl every wfl_j steps (0: none), and with img_frame the frame
 * of step img_it too */
static struct {
    int img_it, wfl_j, img_frame;
    float *image;
    int cut, nb, n1, n2, n3, n1pad, n2pad;
} g_adj = {-1, 0, 0, NULL, 0, 0, 0, 0, 1, 0, 0};

/* snapshot window (cpu programs): per axis (z, x, y) nq samples from padded
 * index f with stride j; frames are cut from the engine's padded frames */
static struct {
    int on;
    int n[3], f[3], j[3], npad[3];
    float *buf;
} g_win;

static void put_frame(const float *frame, size_t n) {
    if (!g_win.on) {
        if (rsf_write(g_wfl, frame, n) != n) die("wfl", "short write");
        return;
    }
    const size_t plane = (size_t)g_win.npad[0] * g_win.npad[1], nout = (size_t)g_win.n[0] * g_win.n[1];
    if (n != plane * g_win.npad[2]) die("wfl", "frame size differs from the padded grid");
    for (int iy = 0; iy < g_win.n[2]; iy++) {
        const float *p = frame + (size_t)(g_win.f[2] + iy * g_win.j[2]) * plane;
        for (int ix = 0; ix < g_win.n[1]; ix++) {
            const float *col = p + (size_t)(g_win.f[1] + ix * g_win.j[1]) * g_win.npad[0] + g_win.f[0];
            float *out = g_win.buf + (size_t)ix * g_win.n[0];
            for (int iz = 0; iz < g_win.n[0]; iz++) out[iz] = col[(size_t)iz * g_win.j[0]];
        }
        if (rsf_write(g_wfl, g_win.buf, nout) != nout) die("wfl", "short write");
    }
}

static void write_frame(void *user, int isnap, int it, const float *frame, size_t n) {
    (void)user;
    (void)isnap;
    if (g_adj.img_it >= 0) {
        if (it == g_adj.img_it) {
            if (!g_adj.cut) {
                memcpy(g_adj.image, frame, n * sizeof(float));
            } else {
                const int nb = g_adj.nb, n3b = g_adj.n3 > 1 ? nb : 0;
                for (int i3 = 0; i3 < g_adj.n3; i3++)
                    for (int i2 = 0; i2 < g_adj.n2; i2++)
                        memcpy(g_adj.image + ((size_t)i3 * g_adj.n2 + i2) * g_adj.n1,
                               frame + ((size_t)(n3b + i3) * g_adj.n2pad + nb + i2) * g_adj.n1pad + nb,
                               sizeof(float) * g_adj.n1);
            }
        }
        const int periodic = g_adj.wfl_j > 0 && it % g_adj.wfl_j == 0;
        const int last = g_adj.img_frame && g_adj.wfl_j > 0 && it == g_adj.img_it;
        if (!periodic && !last) return;
    }
    put_frame(frame, n);
}

int main(int argc, char **argv) {
    rsf_init(argc, argv);
    char name[256];
    snprintf(name, sizeof name, "%s", argv[0]);
    const char *prog = basename(name);
    const int spher = strstr(prog, "spher") != NULL;
    const int ndim = strstr(prog, "3D") != NULL ? 3 : 2;
    const int cart2d = !spher && ndim == 2;
    const int dyn = strstr(prog, "DYNAWEFD") != NULL;
    if (dyn && !(cart2d && strstr(prog, "gpu"))) die(prog, "the moving-geometry program is sfDYNAWEFDcart2Dgpu");
    const int scheme = strstr(prog, "cpu") != NULL ? AWE_SCHEME_CPU : AWE_SCHEME_GPU;
    if (scheme == AWE_SCHEME_CPU && spher) die(prog, "the spherical cpu programs are not provided");
    if (!strstr(prog, "AWEFD")) die(prog, "run as sfAWEFD{cart,spher}{2D,3D}gpu or sfAWEFDcart{2D,3D}cpu");

    /* flags and defaults: MAWEFDcart2Dgpu.cu:74-80, MAWEFDcart3Dgpu.cu:62-68,
     * MAWEFDspher2Dgpu.cu:65-69, MAWEFDspher3Dgpu.cu:88-94,
     * MAWEFDcart{2D,3D}cpu.c:116-128 */
    int fsrf = 0, dabc = 0, snap, bnds, expl, refl = 0, adj = 0, verb = 0, sinc = 0;
    if (scheme == AWE_SCHEME_CPU) {
        snap = bnds = expl = 0;
    } else if (dyn) { /* MDYNAWEFDcart2Dgpu.cu:71-74: no expl/refl (unscaled injection) */
        snap = 1;
        bnds = expl = 0;
    } else {
        snap = cart2d || (spher && ndim == 2);
        bnds = cart2d;
        expl = 1;
        refl = cart2d;
    }
    if (!rsf_get_bool("free", &fsrf) && scheme == AWE_SCHEME_CPU) rsf_get_bool("fsrf", &fsrf);
    rsf_get_bool("dabc", &dabc);
    rsf_get_bool("snap", &snap);
    rsf_get_bool("bnds", &bnds);
    if (!dyn) rsf_get_bool("expl", &expl);
    if (cart2d && scheme == AWE_SCHEME_GPU && !dyn) rsf_get_bool("refl", &refl);
    rsf_get_bool("adj", &adj);
    rsf_get_bool("verb", &verb);
    rsf_get_bool("sinc", &sinc);
    const int spher3 = spher && ndim == 3;
    if (adj && scheme != AWE_SCHEME_CPU && !spher3)
        die(prog, "adj=y (back-injection imaging) is provided for the cpu programs and sfAWEFDspher3Dgpu");
    if (sinc) die(prog, "sinc=y injection is not provided");
    if (dyn) {
        int jd = 1;
        rsf_get_int("jdata", &jd);
        if (jd != 1) die(prog, "jdata must be 1 (the reference writes every step into a buffer of nt/jdata rows)");
    }
    /* snapshot window parameters (read by the cpu programs with snap=y); a
     * given window makes the engine deliver padded frames, which are cut here
     * (2D bnds=y frames are written whole) */
    static const char *win_n[3] = {"nqz", "nqx", "nqy"}, *win_o[3] = {"oqz", "oqx", "oqy"},
                      *win_d[3] = {"dqz", "dqx", "dqy"};
    const int windows = scheme == AWE_SCHEME_CPU && snap;
    int win_given = 0;
    if (windows)
        for (int a = 0; a < ndim; a++)
            win_given |= rsf_get_string(win_n[a]) || rsf_get_string(win_o[a]) || rsf_get_string(win_d[a]);
    g_win.on = win_given && !(ndim == 2 && bnds);
    const char *prec_s = rsf_get_string("precision");
    const int precision = (prec_s && strcmp(prec_s, "exact") == 0) ? AWE_EXACT : AWE_FAST;
    int gpu = 0;
    rsf_get_int("gpu", &gpu);

    rsf_file *Fwav = rsf_input("in"), *Fvel = rsf_input("vel"), *Fsou = rsf_input("sou"), *Frec = rsf_input("rec");
    if (!Fwav || !Fvel || !Fsou || !Frec) die(prog, rsf_error());
    rsf_file *Frfl = NULL, *Fden = NULL;
    if (scheme == AWE_SCHEME_GPU && cart2d && refl && expl) {
        Frfl = rsf_input("rfl");
        if (!Frfl) die(prog, rsf_error());
    }
    int cden = 0;
    rsf_get_bool("cden", &cden);
    if (scheme == AWE_SCHEME_CPU && !cden && rsf_get_string("den")) {
        Fden = rsf_input("den");
        if (!Fden) die(prog, rsf_error());
    }

    /* axes: wavelet n1 = components, n2 = time; model axes 1..ndim */
    const int nt = rsf_n(Fwav, 2), ncs = rsf_n(Fwav, 1);
    const float dt = rsf_d(Fwav, 2), ot = rsf_o(Fwav, 2);
    awe_desc d;
    memset(&d, 0, sizeof d);
    d.coords = spher ? AWE_SPHER : AWE_CART;
    d.scheme = scheme;
    d.ndim = ndim;
    for (int a = 0; a < 3; a++) {
        d.n[a] = a < ndim ? rsf_n(Fvel, a + 1) : 1;
        d.d[a] = a < ndim ? rsf_d(Fvel, a + 1) : 1.f;
        d.o[a] = a < ndim ? rsf_o(Fvel, a + 1) : 0.f;
    }
    d.nb = -1;
    rsf_get_int("nb", &d.nb);
    d.nt = nt;
    d.dt = dt;
    d.jdata = 1;
    rsf_get_int("jdata", &d.jdata);
    d.jsnap = 0;
    if (snap) {
        d.jsnap = nt;
        rsf_get_int("jsnap", &d.jsnap);
    }
    d.bnds = bnds || g_win.on;
    d.fsrf = fsrf;
    d.expl = expl;
    d.refl = refl && expl;
    d.precision = precision;
    if (scheme == AWE_SCHEME_CPU) {
        d.fdorder = 4;
        rsf_get_int("fdorder", &d.fdorder);
        rsf_get_bool("optfd", &d.optfd);
        d.dabc = dabc;
        rsf_get_bool("hybridbc", &d.hybrid);
    }

    /* points: n1 coordinates, count = n2 (* n3 for the programs that read it:
     * MAWEFDcart2Dgpu.cu:120, MAWEFDcart3Dgpu.cu:105, MAWEFDspher2Dgpu.cu:104) */
    const int ncoord = ndim;
    const int use_n3 = scheme == AWE_SCHEME_GPU && !(spher && ndim == 3) && !dyn;
    const int ns = rsf_n(Fsou, 2) * (use_n3 ? rsf_n(Fsou, 3) : 1);
    const int nr = rsf_n(Frec, 2) * (use_n3 ? rsf_n(Frec, 3) : 1);
    /* sfDYNAWEFDcart2Dgpu: n3 = rows of the position tables
     * (MDYNAWEFDcart2Dgpu.cu:103-111), ns*nst and nr*nrt points read */
    const int nst = dyn ? rsf_n(Fsou, 3) : 1, nrt = dyn ? rsf_n(Frec, 3) : 1;
    const size_t nse = (size_t)ns * nst, nre = (size_t)nr * nrt;
    if (rsf_n(Fsou, 1) < ncoord || rsf_n(Frec, 1) < ncoord) die(prog, "sou/rec need one coordinate per axis on n1");
    float *sou = malloc(sizeof(float) * (nse > 0 ? nse : 1) * ncoord);
    float *rec = malloc(sizeof(float) * (nre > 0 ? nre : 1) * ncoord);
    const size_t n1s = (size_t)rsf_n(Fsou, 1), n1r = (size_t)rsf_n(Frec, 1);
    float *tmp = malloc(sizeof(float) * (n1s > n1r ? n1s : n1r));
    for (size_t i = 0; i < nse; i++) {
        if (rsf_read(Fsou, tmp, n1s) != n1s) die(prog, "short read (sou)");
        memcpy(sou + i * ncoord, tmp, sizeof(float) * ncoord);
    }
    for (size_t i = 0; i < nre; i++) {
        if (rsf_read(Frec, tmp, n1r) != n1r) die(prog, "short read (rec)");
        memcpy(rec + i * ncoord, tmp, sizeof(float) * ncoord);
    }
    free(tmp);
    const size_t nmodel = (size_t)d.n[0] * d.n[1] * d.n[2];
    float *vel = malloc(sizeof(float) * nmodel), *rfl = NULL, *den = NULL;
    if (rsf_read(Fvel, vel, nmodel) != nmodel) die(prog, "short read (vel)");
    if (Frfl) {
        rfl = malloc(sizeof(float) * nmodel);
        if (rsf_read(Frfl, rfl, nmodel) != nmodel) die(prog, "short read (rfl)");
    }
    if (Fden) {
        den = malloc(sizeof(float) * nmodel);
        if (rsf_read(Fden, den, nmodel) != nmodel) die(prog, "short read (den)");
    }
    const size_t nwav = (size_t)nt * ncs;
    float *wav = malloc(sizeof(float) * nwav);
    if (rsf_read(Fwav, wav, nwav) != nwav) die(prog, "short read (wavelet)");
    /* the GPU programs inject d_ww[it] for every source; the CPU programs one
     * value per source per step (expl=n) or one for all (expl=y) */
    int wcs = 1;
    if (scheme == AWE_SCHEME_CPU && !expl) wcs = ns;
    if (!adj && wcs > ncs && nwav < (size_t)nt * wcs) die(prog, "wavelet has fewer components than sources");

    /* adj=y: the injected series reversed in time.  The reference seeks to
     * row nt-1-it of the input with the row length it reads: nr traces for
     * the 2D program with expl=n, else the forward row length (ns, or 1 with
     * expl=y). */
    const int img2d = adj && (ndim == 2 || spher3); /* runs that end with an image */
    const int user_jsnap = d.jsnap;
    if (adj) {
        if (img2d) {
            int kt = 0;
            rsf_get_int("kt", &kt);
            if (kt < 1 || kt > nt)
                die(prog, "adj=y: kt must be in [1, nt] (the image is the wavefield of step nt-kt; "
                          "the reference writes none for kt=0)");
            g_adj.img_it = nt - kt;
            d.nt = g_adj.img_it + 1;
        }
        /* sfAWEFDspher3Dgpu reads row nt-1-it with nr samples whatever n1 is */
        const int row = img2d && (spher3 || !expl) ? nr : wcs;
        if (nwav < (size_t)nt * row) die(prog, "adj=y: standard input holds fewer than nt rows");
        float *bw = malloc(sizeof(float) * (size_t)d.nt * row);
        for (int it = 0; it < d.nt; it++)
            memcpy(bw + (size_t)it * row, wav + (size_t)(nt - 1 - it) * row, sizeof(float) * row);
        free(wav);
        wav = bw;
        wcs = row;
    }
    if (img2d) {
        /* frames: the image step, plus the snapshots of snap=y (the engine
         * delivers every gcd(jsnap, nt-kt)-th step and the callback keeps
         * those) */
        g_adj.wfl_j = user_jsnap;
        g_adj.img_frame = spher3;
        int a = user_jsnap > 0 ? user_jsnap : g_adj.img_it, b = g_adj.img_it;
        while (b > 0) {
            const int t = a % b;
            a = b;
            b = t;
        }
        d.jsnap = a > 0 ? a : 1;
        d.jdata = 1;
        if (spher3) d.expl = 0; /* unscaled, as inject_sources_3D_adj */
    }

    awe_plan *plan = NULL;
    if (awe_plan_create(&d, gpu, &plan) != AWE_OK) die(prog, awe_last_error());
    if (awe_set_model(plan, vel, den, scheme == AWE_SCHEME_GPU ? rfl : NULL) != AWE_OK) die(prog, awe_last_error());
    if (img2d) { /* injection at the receivers (expl=n, spherical) or the sources (expl=y); no traces */
        const int at_src = expl && !spher3;
        if (awe_set_geometry(plan, at_src ? ns : nr, at_src ? sou : rec, 0, NULL) != AWE_OK)
            die(prog, awe_last_error());
    } else if (dyn) {
        if (awe_set_moving_geometry(plan, ns, nst, sou, nr, nrt, rec, AWE_MOVE_DYN) != AWE_OK)
            die(prog, awe_last_error());
    } else if (awe_set_geometry(plan, ns, sou, nr, rec) != AWE_OK) {
        die(prog, awe_last_error());
    }
    awe_info info;
    awe_plan_info(plan, &info);
    /* window axes (n, o, d) per axis; 3D bnds=y keeps the window's o and d
     * with the padded n (MAWEFDcart3Dcpu.c:226-233) */
    int wn[3];
    float wo[3], wd[3];
    for (int a = 0; a < 3; a++) {
        wn[a] = d.n[a];
        wo[a] = d.o[a];
        wd[a] = d.d[a];
        if (windows && a < ndim) {
            rsf_get_int(win_n[a], &wn[a]);
            rsf_get_float(win_o[a], &wo[a]);
            rsf_get_float(win_d[a], &wd[a]);
        }
    }
    if (windows && ndim == 3 && bnds)
        for (int a = 0; a < 3; a++) wn[a] = info.npad[a];
    if (g_win.on) {
        static const char *axis[3] = {"z", "x", "y"};
        for (int a = 0; a < 3; a++) {
            const float opad = d.o[a] - (float)info.nbpad * d.d[a];
            int f = a < ndim ? (int)floorf((wo[a] - opad) / d.d[a]) : 0;
            int j = a < ndim ? (int)floorf(wd[a] / d.d[a]) : 0;
            if (bnds && a < 2) { /* whole z-x planes */
                f = 0;
                j = 1;
            }
            const long last = (long)f + (long)(wn[a] - 1) * j;
            if (wn[a] < 1 || f < 0 || j < 0 || last >= info.npad[a]) {
                char msg[160];
                snprintf(msg, sizeof msg, "snapshot window on %s: samples %d..%ld (stride %d) outside the padded "
                         "grid 0..%d", axis[a], f, last, j, info.npad[a] - 1);
                die(prog, msg);
            }
            g_win.n[a] = wn[a];
            g_win.f[a] = f;
            g_win.j[a] = j;
            g_win.npad[a] = info.npad[a];
        }
        g_win.buf = malloc(sizeof(float) * (size_t)g_win.n[0] * g_win.n[1]);
        if (!g_win.buf) die(prog, "out of host memory (snapshot window)");
    }
    if (img2d && windows && (wn[0] != d.n[0] || wn[1] != d.n[1]))
        die(prog, "adj=y: the image is written with the snapshot window's axes, so nqz and nqx must equal the "
                  "model's");
    if (img2d) {
        g_adj.image = calloc((size_t)d.n[0] * d.n[1] * d.n[2], sizeof(float));
        g_adj.cut = d.bnds;
        g_adj.nb = info.nbpad;
        g_adj.n1 = d.n[0];
        g_adj.n2 = d.n[1];
        g_adj.n3 = d.n[2];
        g_adj.n1pad = info.npad[0];
        g_adj.n2pad = info.npad[1];
        if (user_jsnap == 0) awe_set_snapshot_callback(plan, write_frame, NULL);
    }

    rsf_file *Fdat = rsf_output("out");
    if (!Fdat) die(prog, rsf_error());
    if (img2d && spher3) { /* MAWEFDspher3Dgpu.cu:553-555: the model axes */
        rsf_set_axis(Fdat, 1, d.n[0], d.o[0], d.d[0], "ra");
        rsf_set_axis(Fdat, 2, d.n[1], d.o[1], d.d[1], "th");
        rsf_set_axis(Fdat, 3, d.n[2], d.o[2], d.d[2], "ph");
    } else if (img2d) { /* MAWEFDcart2Dcpu.c:362-363: the model axes, or the window's with snap=y */
        rsf_set_axis(Fdat, 1, d.n[0], wo[0], wd[0], "z");
        rsf_set_axis(Fdat, 2, d.n[1], wo[1], wd[1], "x");
    } else {
        rsf_set_axis(Fdat, 1, nr, rsf_o(Frec, 2), rsf_d(Frec, 2), "r");
        rsf_set_axis(Fdat, 2, info.nsmp, ot, dt * d.jdata, "t");
    }
    if (img2d ? user_jsnap > 0 : d.jsnap > 0) {
        g_wfl = rsf_output("wfl");
        if (!g_wfl) die(prog, rsf_error());
        /* snapshot axes as each program writes them: bnds=y keeps the
         * unpadded origin (an sf_setn-only update), except sfAWEFDcart2Dcpu
         * whose padded axes carry the padded origin (MAWEFDcart2Dcpu.c:217-222) */
        const int opad = bnds && scheme == AWE_SCHEME_CPU && ndim == 2;
        float o[3];
        for (int a = 0; a < 3; a++) o[a] = opad ? d.o[a] - info.nbpad * d.d[a] : d.o[a];
        if (spher && ndim == 2) { /* theta fastest */
            rsf_set_axis(g_wfl, 1, bnds ? info.npad[1] : d.n[1], o[1], d.d[1], "th");
            rsf_set_axis(g_wfl, 2, bnds ? info.npad[0] : d.n[0], o[0], d.d[0], "ra");
        } else if (windows && !(ndim == 2 && bnds)) { /* the window's axes */
            const char *lab[3] = {"z", "x", "y"};
            for (int a = 0; a < ndim; a++) rsf_set_axis(g_wfl, a + 1, wn[a], wo[a], wd[a], lab[a]);
        } else {
            const char *lab[2][3] = {{"z", "x", "y"}, {"ra", "th", "ph"}};
            for (int a = 0; a < ndim; a++)
                rsf_set_axis(g_wfl, a + 1, bnds ? info.npad[a] : d.n[a], o[a], d.d[a], lab[spher][a]);
        }
        if (img2d)
            rsf_set_axis(g_wfl, ndim + 1,
                         g_adj.img_it / user_jsnap + 1 + (g_adj.img_frame && g_adj.img_it % user_jsnap != 0), ot,
                         dt * user_jsnap, "t");
        else
            rsf_set_axis(g_wfl, ndim + 1, info.nsnap, ot, dt * d.jsnap, "t");
        awe_set_snapshot_callback(plan, write_frame, NULL);
    }
    float *dat = malloc(sizeof(float) * (size_t)info.nsmp * (nr > 0 ? nr : 1));
    if (verb) fprintf(stderr, "%s: %d steps on a %d x %d x %d padded grid\n", prog, nt, info.npad[0], info.npad[1],
                      info.npad[2]);
    if (awe_forward(plan, wav, wcs, dat, NULL) != AWE_OK) die(prog, awe_last_error());
    if (img2d) {
        const size_t nimg = (size_t)d.n[0] * d.n[1] * d.n[2];
        if (rsf_write(Fdat, g_adj.image, nimg) != nimg) die(prog, "short write (image)");
    } else if (rsf_write(Fdat, dat, (size_t)info.nsmp * nr) != (size_t)info.nsmp * nr) {
        die(prog, "short write (dat)");
    }
    awe_plan_destroy(plan);
    rsf_close(Fdat);
    if (g_wfl) rsf_close(g_wfl);
    rsf_close(Fwav);
    rsf_close(Fvel);
    rsf_close(Fsou);
    rsf_close(Frec);
    if (Frfl) rsf_close(Frfl);
    if (Fden) rsf_close(Fden);
    free(sou);
    free(rec);
    free(vel);
    free(rfl);
    free(den);
    free(wav);
    free(dat);
    free(g_adj.image);
    free(g_win.buf);
    return 0;
}
