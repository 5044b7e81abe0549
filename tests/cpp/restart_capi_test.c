/* The restart-file entry points of include/nsdg.h used from plain C (they
 * are host code and need no GPU): write a restart and a diagnostic file,
 * read both back, check every value, the types, the record count and the
 * error statuses.  Prints "ok" on success; exits non-zero with a message
 * otherwise. */
#include "nsdg.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define CHECK(c)                                                              \
    do {                                                                      \
        if (!(c)) {                                                           \
            fprintf(stderr, "failed at line %d: %s\n", __LINE__, #c);        \
            return 1;                                                         \
        }                                                                     \
    } while (0)

int main(int argc, char** argv)
{
    const char* restart = argc > 1 ? argv[1] : "restart_c.nc";
    const char* diag = argc > 2 ? argv[2] : "diag_c.nc";
    enum { NX = 5, NY = 4, DG = 6 };
    double h[NX * NY * DG], m[NX * NY], back[NX * NY * DG];
    for (int i = 0; i < NX * NY * DG; ++i)
        h[i] = 0.5 + 1e-3 * i;
    for (int i = 0; i < NX * NY; ++i)
        m[i] = (double)(i % 3 != 0);

    nsdg_restart_writer* w = NULL;
    CHECK(nsdg_restart_writer_create(NX, NY, 1, DG, 8, 2, "parametric_rectangular", 3600, "1970-01-01T01:00:00Z",
              &w) == NSDG_OK);
    CHECK(nsdg_restart_writer_add(w, "hice", NSDG_MA_DG, h, NX * NY * DG) == NSDG_OK);
    CHECK(nsdg_restart_writer_add(w, "mask", NSDG_MA_H, m, NX * NY) == NSDG_OK);
    CHECK(nsdg_restart_writer_add(w, "cice", NSDG_MA_DG, h, 7) == NSDG_ERR_SIZE_MISMATCH);
    CHECK(nsdg_restart_writer_save(w, restart) == NSDG_OK);
    nsdg_restart_writer_destroy(w);

    nsdg_restart* r = NULL;
    CHECK(nsdg_restart_open(restart, &r) == NSDG_OK);
    size_t nv = 0;
    CHECK(nsdg_restart_num_vars(r, "data", &nv) == NSDG_OK && nv == 2);
    char name[64], text[128];
    int type = -2;
    size_t nc = 0, nrec = 0, nval = 0;
    CHECK(nsdg_restart_var_info(r, "data", 0, name, sizeof name, &type, &nc, &nrec, &nval) == NSDG_OK);
    CHECK(strcmp(name, "hice") == 0 && type == NSDG_MA_DG && nc == DG && nrec == 1 && nval == NX * NY * DG);
    CHECK(nsdg_restart_read(r, "data/hice", 0, back, NX * NY * DG) == NSDG_OK);
    CHECK(memcmp(back, h, sizeof h) == 0);
    CHECK(nsdg_restart_read(r, "data/hice", 0, back, 3) == NSDG_ERR_SIZE_MISMATCH);
    CHECK(nsdg_restart_read(r, "data/nothere", 0, back, 3) == NSDG_ERR_UNKNOWN_FIELD);
    CHECK(nsdg_restart_dim_names(r, "data/mask", text, sizeof text) == NSDG_OK && strcmp(text, "ydim,xdim") == 0);
    CHECK(nsdg_restart_text(r, "structure", "type", text, sizeof text) == NSDG_OK);
    CHECK(strcmp(text, "parametric_rectangular") == 0);
    CHECK(nsdg_restart_text(r, "metadata/time/time", "formatted", text, 4) == NSDG_ERR_SIZE_MISMATCH);
    nsdg_restart_close(r);

    CHECK(nsdg_diagnostic_writer_create(NX, NY, 1, DG, 8, 2, "parametric_rectangular", 0, "1970-01-01T00:00:00Z",
              &w) == NSDG_OK);
    const char* names[2] = { "hice", "mask" };
    const int types[2] = { NSDG_MA_DG, NSDG_MA_H };
    const size_t counts[2] = { NX * NY * DG, NX * NY };
    for (int rec = 0; rec < 3; ++rec) {
        for (int i = 0; i < NX * NY * DG; ++i)
            h[i] = rec + 1e-3 * i;
        const double* data[2] = { h, m };
        CHECK(nsdg_diagnostic_writer_record(w, 600.0 * rec, 2, names, types, data, counts) == NSDG_OK);
    }
    CHECK(nsdg_restart_writer_save(w, diag) == NSDG_OK);
    nsdg_restart_writer_destroy(w);
    CHECK(nsdg_restart_open(diag, &r) == NSDG_OK);
    CHECK(nsdg_restart_var_info(r, "data", 1, name, sizeof name, &type, &nc, &nrec, &nval) == NSDG_OK);
    CHECK(strcmp(name, "hice") == 0 && nrec == 3 && nval == NX * NY * DG);
    CHECK(nsdg_restart_read(r, "data/hice", 1, back, NX * NY * DG) == NSDG_OK);
    for (int i = 0; i < NX * NY * DG; ++i)
        CHECK(back[i] == 1 + 1e-3 * i);
    CHECK(nsdg_restart_read(r, "data/hice", 3, back, NX * NY * DG) == NSDG_ERR_BAD_ARG);
    nsdg_restart_close(r);

    CHECK(nsdg_restart_open("no_such_file.nc", &r) == NSDG_ERR_BAD_ARG && r == NULL);
    CHECK(strlen(nsdg_restart_last_error(NULL)) > 0);
    printf("ok\n");
    return 0;
}
