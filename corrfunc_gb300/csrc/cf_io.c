/*
 * cf_io.c -- the reference's particle-file readers (io/io.c:29-284, io/ftread.c:22-67), so that
 * command-line programs and C callers can load the same fast-food and ASCII / CSV files.
 *
 * Fast-food ("f"): Fortran unformatted records, each framed by a 4-byte byte count before and
 * after: a header record of 5 ints (idat[1] = number of particles), a record of 9 floats, a
 * record of 1 float, then one record per field holding np values of 4 or 8 bytes.  Values are
 * converted when the file precision differs from the requested one.
 * ASCII ("a") / CSV ("c"): one particle per line, the first num_fields numbers separated by
 * blanks, tabs or commas; lines that do not parse are skipped with a warning.
 * A missing file whose ".gz" version exists is uncompressed with gunzip first, as the
 * reference does.
 */
#define _GNU_SOURCE
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "corrfunc_gb300.h"
#include "cf_internal.h"

/* one framed record of nitems items of size bytes (io/ftread.c:39-67) */
static int ft_record(void *ptr, size_t size, size_t nitems, FILE *fp)
{
    unsigned int n1 = 0, n2 = 0;
    int err = 0;
    if (fread(&n1, sizeof(n1), 1, fp) != 1) {
        fprintf(stderr, "read error, file empty ? \n");
        err = 1;
    }
    const size_t got = fread(ptr, size, nitems, fp);
    if (got != nitems) {
        fprintf(stderr, "read error, %zu items expected, %zu items read. \n", nitems, got);
        err = 1;
    }
    if (fread(&n2, sizeof(n2), 1, fp) != 1) {
        fprintf(stderr, "read error, file too short ? \n");
        err = 1;
    }
    if (n1 != n2) {
        fprintf(stderr, "read warning, byte # do not match, nbyte1 = %u, nbyte2 = %u \n", n1, n2);
        err = 1;
    }
    if (n1 != size * nitems) {
        fprintf(stderr, "read warning, byte # does not match item #, nbyte1 = %u, nitems = %zu \n", n1, nitems);
        err = 1;
    }
    if (err) fprintf(stderr, "ERROR: Read error in ftread while trying to read nitems = %zu of %zu bytes each\n", nitems, size);
    return err ? EXIT_FAILURE : EXIT_SUCCESS;
}

static void free_fields(void **data, int n)
{
    for (int j = 0; j < n; j++) {
        free(data[j]);
        data[j] = NULL;
    }
}

static int64_t read_fastfood(const char *filename, size_t size, int num_fields, void **data)
{
    FILE *fp = fopen(filename, "r");
    if (fp == NULL) {
        fprintf(stderr, "ERROR: Could not open file `%s'\n", filename);
        return -1;
    }
    int idat[5];
    /* header record, then the 9-float and 1-float records skipped unread (io/io.c:113-125) */
    const long skip = (long)(sizeof(int) + 9 * sizeof(float) + sizeof(int) + sizeof(int) + sizeof(float) + sizeof(int));
    if (ft_record(idat, sizeof(int), 5, fp) != EXIT_SUCCESS || fseek(fp, skip, SEEK_CUR) != 0) {
        fclose(fp);
        return -1;
    }
    const int64_t np = idat[1];
    if (np < 0) {
        fclose(fp);
        return -1;
    }
    unsigned int nbytes = 0;
    if (fread(&nbytes, sizeof(nbytes), 1, fp) != 1 || fseek(fp, -4, SEEK_CUR) != 0) {
        fclose(fp);
        return -1;
    }
    const unsigned int fsize = np > 0 ? (unsigned int)(nbytes / (uint64_t)np) : (unsigned int)size;
    if (fsize != 4 && fsize != 8) {
        fprintf(stderr, "Data-type in file = %u must be either 4 byte (float) or 8 byte(double) precision\n", fsize);
        fclose(fp);
        return -1;
    }
    if (fsize != size)
        fprintf(stderr, "WARNING: File was written in a different precision than requested (file precision = %u "
                "requested precision = %zu)\n", fsize, size);
    void *tmp = fsize != size ? malloc((size_t)fsize * (size_t)(np > 0 ? np : 1)) : NULL;
    for (int i = 0; i < num_fields; i++) {
        data[i] = malloc(size * (size_t)(np > 0 ? np : 1));
        if (data[i] == NULL || (fsize != size && tmp == NULL)) {
            free_fields(data, i + 1);
            free(tmp);
            fclose(fp);
            return -1;
        }
        void *dst = fsize == size ? data[i] : tmp;
        if (ft_record(dst, fsize, (size_t)np, fp) != EXIT_SUCCESS) {
            free_fields(data, i + 1);
            free(tmp);
            fclose(fp);
            return -1;
        }
        if (fsize == 4 && size == 8)
            for (int64_t j = 0; j < np; j++) ((double *)data[i])[j] = ((const float *)tmp)[j];
        else if (fsize == 8 && size == 4)
            for (int64_t j = 0; j < np; j++) ((float *)data[i])[j] = (float)((const double *)tmp)[j];
    }
    free(tmp);
    fclose(fp);
    return np;
}

static int64_t read_ascii(const char *filename, size_t size, int num_fields, void **data)
{
    FILE *fp = fopen(filename, "r");
    if (fp == NULL) {
        fprintf(stderr, "ERROR: Could not open file `%s'\n", filename);
        return -1;
    }
    int64_t cap = 300000, n = 0;
    for (int j = 0; j < num_fields; j++) {
        data[j] = malloc(size * (size_t)cap);
        if (data[j] == NULL) {
            free_fields(data, j);
            fclose(fp);
            return -1;
        }
    }
    char buf[10000];
    while (fgets(buf, sizeof buf, fp) != NULL) {
        char *save = NULL, *copy = buf;
        int ok = 1;
        for (int j = 0; j < num_fields; j++, copy = NULL) {
            const char *tok = strtok_r(copy, " ,\t", &save);
            double v;
            if (tok != NULL && sscanf(tok, "%lf", &v) == 1) {
                if (size == 4) ((float *)data[j])[n] = (float)v;
                else ((double *)data[j])[n] = v;
            } else {
                ok = 0;
            }
        }
        if (ok) {
            n++;
        } else {
            fprintf(stderr, "io> WARNING: Could not parse all requested %d fields in line %lld. Skipping that line\n",
                    num_fields, (long long)n);
        }
        if (n == cap) {
            cap = cap + cap / 10 + 5;
            for (int j = 0; j < num_fields; j++) {
                void *p = realloc(data[j], size * (size_t)cap);
                if (p == NULL) {
                    free_fields(data, num_fields);
                    fclose(fp);
                    return -1;
                }
                data[j] = p;
            }
        }
    }
    fclose(fp);
    for (int j = 0; j < num_fields; j++) {
        void *p = realloc(data[j], size * (size_t)(n > 0 ? n : 1));
        if (p != NULL) data[j] = p;
    }
    return n;
}

int64_t read_columns_into_array(const char *filename, const char *format, const size_t size, const int num_fields,
                                void **data)
{
    if (num_fields < 1) {
        fprintf(stderr, "Number of fields to read-in = %d must be at least 1\n", num_fields);
        return -1;
    }
    if (size != 4 && size != 8) {
        fprintf(stderr, "Size of fields = %zu must be either 4 or 8\n", size);
        return -1;
    }
    if (filename == NULL || format == NULL) return -1;
    FILE *probe = fopen(filename, "r");
    if (probe == NULL) {
        char gz[4096];
        snprintf(gz, sizeof gz, "%s.gz", filename);
        FILE *g = fopen(gz, "r");
        if (g == NULL) {
            fprintf(stderr, "ERROR: Could not find file: neither as `%s' nor as `%s'\n", filename, gz);
            return -1;
        }
        fclose(g);
        char cmd[8192];
        snprintf(cmd, sizeof cmd, "gunzip '%s.gz'", filename);
        fprintf(stderr, "Could not locate `%s' but found the gzip file `%s.gz'.\nRunning system command `%s' now to "
                "uncompress\n", filename, filename, cmd);
        if (system(cmd) != 0) return -1;
    } else {
        fclose(probe);
    }
    if (strncmp(format, "f", 1) == 0) return read_fastfood(filename, size, num_fields, data);
    if (strncmp(format, "a", 1) == 0 || strncmp(format, "c", 1) == 0) return read_ascii(filename, size, num_fields, data);
    fprintf(stderr, "ERROR: In %s> Unknown format `%s'\n", __func__, format);
    return -1;
}

int64_t read_positions(const char *filename, const char *format, const size_t size, const int num_fields, ...)
{
    if (num_fields < 1) {
        fprintf(stderr, "Number of fields to read-in = %d must be at least 1\n", num_fields);
        return -1;
    }
    void **cols = calloc((size_t)num_fields, sizeof(void *));
    if (cols == NULL) return -1;
    const int64_t np = read_columns_into_array(filename, format, size, num_fields, cols);
    va_list ap;
    va_start(ap, num_fields);
    for (int i = 0; i < num_fields; i++) {
        void **dst = va_arg(ap, void **);
        *dst = np >= 0 ? cols[i] : NULL;
    }
    va_end(ap);
    free(cols);
    return np;
}

/* Extension: the same read, then each field copied into a new device buffer (released with
 * cf_gpu_free_device), for callers of cf_gpu_countpairs_device.  The host copies are freed. */
int64_t cf_gpu_read_positions_device(const char *filename, const char *format, const size_t size, const int num_fields,
                                     void **device_fields)
{
    if (num_fields < 1 || device_fields == NULL) return -1;
    void **cols = calloc((size_t)num_fields, sizeof(void *));
    if (cols == NULL) return -1;
    const int64_t np = read_columns_into_array(filename, format, size, num_fields, cols);
    int ok = np >= 0;
    for (int i = 0; i < num_fields; i++) {
        device_fields[i] = NULL;
        if (ok && cf_engine_to_device(cols[i], size * (size_t)(np > 0 ? np : 1), &device_fields[i]) != EXIT_SUCCESS) ok = 0;
    }
    for (int i = 0; i < num_fields; i++) free(cols[i]);
    free(cols);
    if (!ok) {
        for (int i = 0; i < num_fields; i++) {
            cf_gpu_free_device(device_fields[i]);
            device_fields[i] = NULL;
        }
        return -1;
    }
    return np;
}

void cf_gpu_free_device(void *device_ptr) { cf_engine_free_device(device_ptr); }
