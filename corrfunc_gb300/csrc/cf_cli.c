/*
 * cf_cli.c -- the reference's command-line programs, one multi-call binary (the command is the
 * name it is run as): DD, DDrppi, DDsmu, wp, xi, vpf (theory/<name>/<name>.c) and DDtheta_mocks,
 * DDrppi_mocks, DDsmu_mocks, vpf_mocks (mocks/<name>/<name>.c).  Same positional arguments
 * (the OpenMP builds' argument lists, numthreads included), same optional weight arguments, same
 * stdout table formats, same exit codes; the counting runs on the GPU library.
 *
 * Options follow the reference's default builds (theory.options, mocks.options, common.mk):
 * theory programs count periodically without separation averages and read positions in single
 * precision; the mocks programs read double precision and output the averages.  Setting
 * CF_CLI_DOUBLE=1 in the environment reads the theory programs' inputs in double precision
 * instead (the reference built with DOUBLE_PREC).
 */
#define _GNU_SOURCE
#include <inttypes.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include "corrfunc_gb300.h"

static double now_s(void)
{
    struct timeval t;
    gettimeofday(&t, NULL);
    return t.tv_sec + 1e-6 * t.tv_usec;
}

static void usage(const char *cmd, const char *const *names, int n, const char *const *opt, int nopt, int argc,
                  char **argv)
{
    fprintf(stderr, "=========================================================================\n");
    fprintf(stderr, "   --- %s", cmd);
    for (int i = 0; i < n; i++) fprintf(stderr, " %s", names[i]);
    if (nopt) {
        fprintf(stderr, " [");
        for (int i = 0; i < nopt; i++) fprintf(stderr, "%s%s", i ? " " : "", opt[i]);
        fprintf(stderr, "]");
    }
    fprintf(stderr, "\n=========================================================================\n");
    fprintf(stderr, "\nFound: %d parameters\n ", argc - 1);
    for (int i = 1; i < argc; i++)
        fprintf(stderr, "\t\t %s = `%s' \n", i <= n ? names[i - 1] : (i <= n + nopt ? opt[i - 1 - n] : "<>"), argv[i]);
    for (int i = argc; i <= n; i++) fprintf(stderr, "\t\t %s = `?'\n", names[i - 1]);
}

/* positional arguments and the optional weight block (0, 3 or 5 extra arguments for two sets,
 * 0 or 3 for one) */
static int check_args(const char *cmd, const char *const *names, int n, int two_sets, int argc, char **argv)
{
    static const char *const opt2[] = {"weight_method", "weights_file1", "weights_format1", "weights_file2",
                                       "weights_format2"};
    const int nopt = two_sets ? 5 : 3;
    if (argc < n + 1) {
        usage(cmd, names, n, opt2, nopt, argc, argv);
        fprintf(stderr, "\nMissing required parameters \n");
        return -1;
    }
    const int given = argc - (n + 1);
    if (!(given == 0 || given == 3 || (two_sets && given == 5))) {
        usage(cmd, names, n, opt2, nopt, argc, argv);
        fprintf(stderr, "\nFound: %d optional arguments; must be 0 (no weights), 3 (for one set of weights)%s\n ", given,
                two_sets ? " or 5 (for two sets)" : "");
        return -1;
    }
    fprintf(stderr, "Running `%s' with the parameters \n\n\t\t -------------------------------------\n", argv[0]);
    for (int i = 1; i < argc; i++)
        fprintf(stderr, "\t\t %-10s = %s \n", i <= n ? names[i - 1] : opt2[i - 1 - n], argv[i]);
    fprintf(stderr, "\t\t -------------------------------------\n");
    return given;
}

typedef struct {
    int64_t n;
    void *c[3];
    void *w[MAX_NUM_WEIGHTS];
} cli_set;

static void set_free(cli_set *s)
{
    for (int k = 0; k < 3; k++) free(s->c[k]);
    for (int k = 0; k < MAX_NUM_WEIGHTS; k++) free(s->w[k]);
    memset(s, 0, sizeof(*s));
}

static int read_set(const char *file, const char *fmt, size_t es, int nfields, const char *wfile, const char *wfmt,
                    int nw, cli_set *s)
{
    memset(s, 0, sizeof(*s));
    s->n = read_columns_into_array(file, fmt, es, nfields, s->c);
    if (s->n < 0) return -1;
    if (wfile != NULL && nw > 0) {
        const int64_t m = read_columns_into_array(wfile, wfmt, es, nw, s->w);
        if (m != s->n) {
            fprintf(stderr, "Error: read %" PRId64 " lines from %s, but read %" PRId64 " from %s\n", m, wfile, s->n, file);
            return -1;
        }
    }
    return 0;
}

/* weight method and its files for set 1 / set 2 */
typedef struct {
    weight_method_t method;
    int nw;
    const char *f1, *fmt1, *f2, *fmt2;
} cli_weights;

static int parse_weights(int given, int n, char **argv, cli_weights *W)
{
    memset(W, 0, sizeof(*W));
    W->method = NONE;
    if (given >= 3) {
        if (get_weight_method_by_name(argv[n + 1], &W->method) != EXIT_SUCCESS) {
            fprintf(stderr, "Error: Unknown weight method \"%s\"\n", argv[n + 1]);
            return -1;
        }
        W->nw = get_num_weights_by_method(W->method);
        W->f1 = argv[n + 2];
        W->fmt1 = argv[n + 3];
    }
    if (given >= 5) {
        W->f2 = argv[n + 4];
        W->fmt2 = argv[n + 5];
    }
    return 0;
}

static struct extra_options extra_for(const cli_weights *W, cli_set *a, cli_set *b)
{
    struct extra_options e = get_extra_options(W->method);
    for (int k = 0; k < W->nw; k++) {
        e.weights0.weights[k] = a->w[k];
        e.weights1.weights[k] = b->w[k];
    }
    return e;
}

static size_t theory_size(void)
{
    const char *d = getenv("CF_CLI_DOUBLE");
    return (d && d[0] == '1') ? sizeof(double) : sizeof(float);
}

static double parse_real(const char *s, size_t es)
{
    double v = atof(s);
    return es == sizeof(float) ? (double)(float)v : v;
}

/* theory options of the default build: periodic, no averages, the host's fastest formula */
static struct config_options theory_options(size_t es, double boxsize)
{
    struct config_options o = get_config_options();
    o.float_type = es;
    o.periodic = 1;
    o.need_avg_sep = 0;
    o.verbose = 1;
    o.boxsize_x = boxsize;
    o.boxsize_y = BOXSIZE_NOTGIVEN;
    o.boxsize_z = BOXSIZE_NOTGIVEN;
    return o;
}

static struct config_options mocks_options(void)
{
    struct config_options o = get_config_options();
    o.float_type = sizeof(double);
    o.periodic = 0;
    o.need_avg_sep = 1;
    o.verbose = 1;
    o.link_in_dec = 1;
    o.link_in_ra = 1;
    return o;
}

/* two-set pair counters: DD, DDrppi, DDsmu, DDtheta_mocks, DDrppi_mocks, DDsmu_mocks */
static int run_pairs(const char *cmd, int argc, char **argv)
{
    const int is_dd = !strcmp(cmd, "DD"), is_rppi = !strcmp(cmd, "DDrppi"), is_smu = !strcmp(cmd, "DDsmu");
    const int is_theta = !strcmp(cmd, "DDtheta_mocks"), is_rppi_m = !strcmp(cmd, "DDrppi_mocks");
    const int mocks = is_theta || is_rppi_m || !strcmp(cmd, "DDsmu_mocks");
    static const char *const n_dd[] = {"file1", "format1", "file2", "format2", "binfile", "boxsize", "Nthreads"};
    static const char *const n_rppi[] = {"file1", "format1", "file2", "format2", "binfile", "pimax", "boxsize",
                                         "Nthreads"};
    static const char *const n_smu[] = {"file1", "format1", "file2", "format2", "sbinfile", "mu_max", "nmu_bins",
                                        "boxsize", "Nthreads"};
    static const char *const n_theta[] = {"file1", "format1", "file2", "format2", "binfile", "Nthreads"};
    static const char *const n_rppi_m[] = {"file1", "format1", "file2", "format2", "binfile", "pimax",
                                           "cosmology flag", "numthreads"};
    static const char *const n_smu_m[] = {"file1", "format1", "file2", "format2", "sbinfile", "mu_max", "nmu_bins",
                                          "cosmology flag", "numthreads"};
    const char *const *names = is_dd ? n_dd : is_rppi ? n_rppi : is_smu ? n_smu : is_theta ? n_theta
                                                                             : is_rppi_m ? n_rppi_m : n_smu_m;
    const int n = is_dd ? 7 : is_rppi ? 8 : is_smu ? 9 : is_theta ? 6 : is_rppi_m ? 8 : 9;
    const double t_start = now_s();
    const int given = check_args(cmd, names, n, 1, argc, argv);
    if (given < 0) return EXIT_FAILURE;
    const int nthreads = atoi(argv[n]);
    if (nthreads < 1) {
        fprintf(stderr, "Error: Nthreads must be at least 1...returning\n");
        return EXIT_FAILURE;
    }
    cli_weights W;
    if (parse_weights(given, n, argv, &W) != 0) return EXIT_FAILURE;
    const size_t es = mocks ? sizeof(double) : theory_size();
    const int nf = is_theta ? 2 : 3;
    const int autocorr = strcmp(argv[1], argv[3]) == 0;
    double t0 = now_s();
    cli_set a, b;
    memset(&b, 0, sizeof(b));
    if (read_set(argv[1], argv[2], es, nf, W.f1, W.fmt1, W.nw, &a) != 0) return EXIT_FAILURE;
    if (!autocorr && read_set(argv[3], argv[4], es, nf, W.f2, W.fmt2, W.nw, &b) != 0) return EXIT_FAILURE;
    cli_set *s2 = autocorr ? &a : &b;
    const double read_time = now_s() - t0;
    struct extra_options extra = extra_for(&W, &a, s2);
    t0 = now_s();
    int rc;
    if (is_dd || is_rppi || is_smu) {
        const double boxsize = atof(argv[is_dd ? 6 : is_rppi ? 7 : 8]);
        struct config_options o = theory_options(es, boxsize);
        if (is_dd) {
            results_countpairs r;
            rc = countpairs(a.n, a.c[0], a.c[1], a.c[2], s2->n, s2->c[0], s2->c[1], s2->c[2], nthreads, autocorr,
                            argv[5], &r, &o, &extra);
            if (rc == EXIT_SUCCESS) {
                double rlow = r.rupp[0];
                for (int i = 1; i < r.nbin; i++) {
                    fprintf(stdout, "%e\t%e\t%e\t%12" PRIu64 "\t%e\n", rlow, r.rupp[i], r.rpavg[i], r.npairs[i],
                            r.weightavg[i]);
                    rlow = r.rupp[i];
                }
                free_results(&r);
            }
        } else if (is_rppi) {
            const double pimax = parse_real(argv[6], es);
            results_countpairs_rp_pi r;
            rc = countpairs_rp_pi(a.n, a.c[0], a.c[1], a.c[2], s2->n, s2->c[0], s2->c[1], s2->c[2], nthreads,
                                  autocorr, argv[5], pimax, &r, &o, &extra);
            if (rc == EXIT_SUCCESS) {
                const double dpi = pimax / (double)r.npibin;
                for (int i = 1; i < r.nbin; i++) {
                    const double logrp = log10(r.rupp[i]);
                    for (int j = 0; j < r.npibin; j++) {
                        const int k = i * (r.npibin + 1) + j;
                        fprintf(stdout, "%e\t%e\t%e\t%12" PRIu64 "\t%e\n", logrp, (j + 1) * dpi, r.rpavg[k], r.npairs[k],
                                r.weightavg[k]);
                    }
                }
                free_results_rp_pi(&r);
            }
        } else {
            const double mu_max = atof(argv[6]);
            const int nmu = atoi(argv[7]);
            results_countpairs_s_mu r;
            rc = countpairs_s_mu(a.n, a.c[0], a.c[1], a.c[2], s2->n, s2->c[0], s2->c[1], s2->c[2], nthreads, autocorr,
                                 argv[5], mu_max, nmu, &r, &o, &extra);
            if (rc == EXIT_SUCCESS) {
                double smin = r.supp[0];
                const double dmu = mu_max / (double)nmu;
                for (int i = 1; i < r.nsbin; i++) {
                    for (int j = 0; j < nmu; j++) {
                        const int k = i * (nmu + 1) + j;
                        fprintf(stdout, "%e\t%e\t%e\t%12" PRIu64 "\t%e\n", smin, r.supp[i], (j + 1) * dmu, r.npairs[k],
                                r.weightavg[k]);
                    }
                    smin = r.supp[i];
                }
                free_results_s_mu(&r);
            }
        }
    } else {
        struct config_options o = mocks_options();
        if (is_theta) {
            results_countpairs_theta r;
            rc = countpairs_theta_mocks(a.n, a.c[0], a.c[1], s2->n, s2->c[0], s2->c[1], nthreads, autocorr, argv[5], &r,
                                        &o, &extra);
            if (rc == EXIT_SUCCESS) {
                double tlow = r.theta_upp[0];
                for (int i = 1; i < r.nbin; i++) {
                    fprintf(stdout, "%20.8lf %20.8lf %20.8lf %10" PRIu64 " %20.8lf\n", tlow, r.theta_upp[i],
                            r.theta_avg[i], r.npairs[i], r.weightavg[i]);
                    tlow = r.theta_upp[i];
                }
                free_results_countpairs_theta(&r);
            }
        } else if (is_rppi_m) {
            const double pimax = atof(argv[6]);
            const int cosmology = atoi(argv[7]);
            results_countpairs_mocks r;
            rc = countpairs_mocks(a.n, a.c[0], a.c[1], a.c[2], s2->n, s2->c[0], s2->c[1], s2->c[2], nthreads, autocorr,
                                  argv[5], pimax, cosmology, &r, &o, &extra);
            if (rc == EXIT_SUCCESS) {
                const double dpi = pimax / (double)r.npibin;
                for (int i = 1; i < r.nbin; i++) {
                    const double logrp = log10(r.rupp[i]);
                    for (int j = 0; j < r.npibin; j++) {
                        const int k = i * (r.npibin + 1) + j;
                        fprintf(stdout, "%10" PRIu64 " %20.8lf %20.8lf  %20.8lf %20.8lf \n", r.npairs[k], r.rpavg[k],
                                logrp, (j + 1) * dpi, r.weightavg[k]);
                    }
                }
                free_results_mocks(&r);
            }
        } else {
            const double mu_max = atof(argv[6]);
            const int nmu = atoi(argv[7]);
            const int cosmology = atoi(argv[8]);
            results_countpairs_mocks_s_mu r;
            rc = countpairs_mocks_s_mu(a.n, a.c[0], a.c[1], a.c[2], s2->n, s2->c[0], s2->c[1], s2->c[2], nthreads,
                                       autocorr, argv[5], mu_max, nmu, cosmology, &r, &o, &extra);
            if (rc == EXIT_SUCCESS) {
                const double dmu = mu_max / (double)r.nmu_bins;
                for (int i = 1; i < r.nsbin; i++) {
                    const double logs = log10(r.supp[i]);
                    for (int j = 0; j < r.nmu_bins; j++) {
                        const int k = i * (r.nmu_bins + 1) + j;
                        fprintf(stdout, "%10" PRIu64 " %20.8lf %20.8lf  %20.8lf %20.8lf \n", r.npairs[k], r.savg[k],
                                logs, (j + 1) * dmu, r.weightavg[k]);
                    }
                }
                free_results_mocks_s_mu(&r);
            }
        }
    }
    const double pair_time = now_s() - t0;
    const int64_t n1 = a.n, n2 = s2->n;
    set_free(&a);
    if (!autocorr) set_free(&b);
    if (rc != EXIT_SUCCESS) return rc;
    fprintf(stderr, "%s> Done -  ND1=%" PRId64 " ND2=%" PRId64 ". Time taken = %6.2lf seconds. read-in time = %6.2lf seconds "
            "sec pair-counting time = %6.2lf sec\n", cmd, n1, n2, now_s() - t_start, read_time, pair_time);
    return EXIT_SUCCESS;
}

/* one-set box counters: wp, xi */
static int run_box(const char *cmd, int argc, char **argv)
{
    const int is_wp = !strcmp(cmd, "wp");
    static const char *const n_wp[] = {"boxsize", "file", "format", "binfile", "pimax", "Nthreads"};
    static const char *const n_xi[] = {"boxsize", "file", "format", "binfile", "Nthreads"};
    const int n = is_wp ? 6 : 5;
    const double t_start = now_s();
    const int given = check_args(cmd, is_wp ? n_wp : n_xi, n, 0, argc, argv);
    if (given < 0) return EXIT_FAILURE;
    const int nthreads = atoi(argv[n]);
    if (nthreads < 1) {
        fprintf(stderr, "Error: Nthreads must be at least 1...returning\n");
        return EXIT_FAILURE;
    }
    cli_weights W;
    if (parse_weights(given, n, argv, &W) != 0) return EXIT_FAILURE;
    const size_t es = theory_size();
    cli_set a;
    if (read_set(argv[2], argv[3], es, 3, W.f1, W.fmt1, W.nw, &a) != 0) return EXIT_FAILURE;
    const double boxsize = atof(argv[1]);
    struct extra_options extra = extra_for(&W, &a, &a);
    struct config_options o = theory_options(es, boxsize);
    int rc;
    if (is_wp) {
        const double pimax = parse_real(argv[5], es);
        results_countpairs_wp r;
        rc = countpairs_wp(a.n, a.c[0], a.c[1], a.c[2], boxsize, nthreads, argv[4], pimax, &r, &o, &extra);
        if (rc == EXIT_SUCCESS) {
            double rlow = r.rupp[0];
            for (int i = 1; i < r.nbin; i++) {
                fprintf(stdout, "%e\t%e\t%e\t%12" PRIu64 "\t%e\t%e\n", rlow, r.rupp[i], r.rpavg[i], r.npairs[i], r.wp[i],
                        r.weightavg[i]);
                rlow = r.rupp[i];
            }
            free_results_wp(&r);
        }
    } else {
        results_countpairs_xi r;
        rc = countpairs_xi(a.n, a.c[0], a.c[1], a.c[2], boxsize, nthreads, argv[4], &r, &o, &extra);
        if (rc == EXIT_SUCCESS) {
            double rlow = r.rupp[0];
            for (int i = 1; i < r.nbin; i++) {
                fprintf(stdout, "%e\t%e\t%e\t%12" PRIu64 "\t%e\t%e\n", rlow, r.rupp[i], r.ravg[i], r.npairs[i], r.xi[i],
                        r.weightavg[i]);
                rlow = r.rupp[i];
            }
            free_results_xi(&r);
        }
    }
    const int64_t np = a.n;
    set_free(&a);
    if (rc != EXIT_SUCCESS) return rc;
    fprintf(stderr, "%s> Done -  ND1=%" PRId64 ". Time taken = %6.2lf seconds.\n", cmd, np, now_s() - t_start);
    return EXIT_SUCCESS;
}

static void print_pn(double **pN, int nbin, int num_pN, double rmax, int mocks)
{
    const double rstep = rmax / (double)nbin;
    for (int b = 0; b < nbin; b++) {
        const double r = (b + 1) * rstep;
        if (mocks) fprintf(stdout, "%10.2lf ", r);
        else fprintf(stdout, "%lf ", r);
        for (int i = 0; i < num_pN; i++) fprintf(stdout, " %10.4e", pN[b][i]);
        fprintf(stdout, "\n");
    }
}

/* theory/vpf/vpf.c: rmax nbins ncentres num_pN file format seed boxsize */
static int run_vpf(int argc, char **argv)
{
    static const char *const names[] = {"rmax", "nbins", "ncentres", "num_pN", "file", "format", "seed", "boxsize"};
    const double t_start = now_s();
    if (argc < 9) {
        usage("vpf", names, 8, NULL, 0, argc, argv);
        fprintf(stderr, "\nMissing required parameters \n");
        return EXIT_FAILURE;
    }
    const double rmax = atof(argv[1]);
    const int nbin = atoi(argv[2]), nc = atoi(argv[3]), num_pN = atoi(argv[4]);
    const unsigned long seed = (unsigned long)atol(argv[7]);
    const size_t es = theory_size();
    cli_set a;
    if (read_set(argv[5], argv[6], es, 3, NULL, NULL, 0, &a) != 0) return EXIT_FAILURE;
    struct config_options o = theory_options(es, atof(argv[8]));
    results_countspheres r;
    const int rc = countspheres(a.n, a.c[0], a.c[1], a.c[2], rmax, nbin, nc, num_pN, seed, &r, &o, NULL);
    const int64_t np = a.n;
    set_free(&a);
    if (rc != EXIT_SUCCESS) return rc;
    print_pn(r.pN, r.nbin, num_pN, rmax, 0);
    free_results_countspheres(&r);
    fprintf(stderr, "vpf> Done. Ngal = %" PRId64 ". Time taken = %0.2lf seconds \n", np, now_s() - t_start);
    return EXIT_SUCCESS;
}

/* mocks/vpf_mocks/vpf_mocks.c: rmax nbin ncenters num_pN volume galaxy-file format randoms-file
 * format centers-file cosmology; the randoms' neighbour threshold is N_expected - sqrt(N_expected)
 * (mocks/vpf_mocks/vpf_mocks.c:140-150) */
static int run_vpf_mocks(int argc, char **argv)
{
    static const char *const names[] = {"rmax", "nbin", "ncenters", "num_pN", "volume", "galaxy file",
                                        "galaxy file-format", "randoms file", "randoms file-format", "centers file",
                                        "cosmology flag"};
    const double t_start = now_s();
    if (argc < 12) {
        usage("vpf_mocks", names, 11, NULL, 0, argc, argv);
        fprintf(stderr, "\nMissing required parameters \n");
        return EXIT_FAILURE;
    }
    const double rmax = atof(argv[1]), volume = atof(argv[5]);
    const int nbin = atoi(argv[2]), nc = atoi(argv[3]), num_pN = atoi(argv[4]), cosmology = atoi(argv[11]);
    const char *centers = argv[10];
    if (!(rmax > 0) || nbin <= 0 || nc <= 0) {
        fprintf(stderr, "invalid rmax / nbin / ncenters\n");
        return EXIT_FAILURE;
    }
    int need_randoms = 1;
    FILE *fp = fopen(centers, "r");
    if (fp != NULL) {
        double rr = 0.0;
        const int nread = fscanf(fp, "%*f %*f %*f %lf", &rr);
        fclose(fp);
        if (nread == 1 && rr >= rmax) {
            /* count the centres (lines that are not comments) */
            FILE *f2 = fopen(centers, "r");
            char line[10000];
            int64_t lines = 0;
            while (f2 && fgets(line, sizeof line, f2)) {
                const char *c = line;
                while (*c == ' ' || *c == '\t' || *c == '\n' || *c == '\r') c++;
                if (*c && *c != '#') lines++;
            }
            if (f2) fclose(f2);
            if (lines >= nc) need_randoms = 0;
        }
    }
    cli_set g, rnd;
    memset(&rnd, 0, sizeof(rnd));
    if (read_set(argv[6], argv[7], sizeof(double), 3, NULL, NULL, 0, &g) != 0) return EXIT_FAILURE;
    int threshold = 1;
    int64_t nran = nc;
    if (need_randoms) {
        if (read_set(argv[8], argv[9], sizeof(double), 3, NULL, NULL, 0, &rnd) != 0) return EXIT_FAILURE;
        if (!(volume > 0)) {
            fprintf(stderr, "Mock volume must be > 0\n");
            return EXIT_FAILURE;
        }
        const double nexp = (double)rnd.n * (4.0 * M_PI * (rmax * rmax * rmax) / 3.) / volume;
        threshold = (int)(nexp - sqrt(nexp));
        nran = rnd.n;
    }
    struct config_options o = mocks_options();
    results_countspheres_mocks r;
    const int rc = countspheres_mocks(g.n, g.c[0], g.c[1], g.c[2], nran, rnd.c[0], rnd.c[1], rnd.c[2], threshold, rmax,
                                      nbin, nc, num_pN, centers, cosmology, &r, &o, NULL);
    const int64_t ng = g.n;
    set_free(&g);
    set_free(&rnd);
    if (rc != EXIT_SUCCESS) return rc;
    print_pn(r.pN, r.nbin, num_pN, rmax, 1);
    free_results_countspheres_mocks(&r);
    fprintf(stderr, "vpf_mocks> Done. Ngal = %" PRId64 ". Time taken = %0.2lf seconds \n", ng, now_s() - t_start);
    return EXIT_SUCCESS;
}

int main(int argc, char **argv)
{
    const char *cmd = strrchr(argv[0], '/');
    cmd = cmd ? cmd + 1 : argv[0];
    if (!strcmp(cmd, "DD") || !strcmp(cmd, "DDrppi") || !strcmp(cmd, "DDsmu") || !strcmp(cmd, "DDtheta_mocks") ||
        !strcmp(cmd, "DDrppi_mocks") || !strcmp(cmd, "DDsmu_mocks"))
        return run_pairs(cmd, argc, argv);
    if (!strcmp(cmd, "wp") || !strcmp(cmd, "xi")) return run_box(cmd, argc, argv);
    if (!strcmp(cmd, "vpf")) return run_vpf(argc, argv);
    if (!strcmp(cmd, "vpf_mocks")) return run_vpf_mocks(argc, argv);
    fprintf(stderr, "%s: run as one of DD, DDrppi, DDsmu, wp, xi, vpf, DDtheta_mocks, DDrppi_mocks, DDsmu_mocks, "
            "vpf_mocks (the programs in corrfunc_gb300/bin are links to this binary)\n", cmd);
    return EXIT_FAILURE;
}
