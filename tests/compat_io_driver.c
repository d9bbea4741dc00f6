/*
 * compat_io_driver.c -- test program for the readers and run_bc of
 * libgbsssp_compat.so, called the way main/main.c:207-231 calls the
 * reference's: scan_csr_idx + read_graph_csr, read_csr_bin, run_bc.
 *
 *   compat_io_driver text|bin DIR FILE TYPE OUT
 *       OUT: int64 v_size, e_size, offset, global_v_size; per vertex int64
 *       vet_idx and double weight, wb, recip and int64 vet_deg; per edge int64
 *       edge_idx and double edge_weight.
 *   compat_io_driver bc DIR FILE [bin]
 *       run_bc's printout on stdout.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gbsssp_compat.h"

int bin = 0;   /* the reference's global flag (main/main.c:18) */

int main(int argc, char **argv) {
    if (argc < 4) return 2;
    gbs_compat_set_exit(0);
    if (!strcmp(argv[1], "bc")) {
        bin = argc > 4 && !strcmp(argv[4], "bin");
        run_bc(argv[3], argv[2]);
        return gbs_compat_status() == GBS_OK ? 0 : 1;
    }
    if (argc < 6) return 2;
    t_csr *gs = (t_csr *)calloc(1, sizeof(t_csr));
    sint type = (sint)atoi(argv[4]);
    if (!strcmp(argv[1], "text")) {
        scan_csr_idx(gs, argv[3], argv[2], type);
        if (gbs_compat_status() != GBS_OK) return 1;
        read_graph_csr(gs, argv[3], argv[2], type);
    } else {
        read_csr_bin(gs, argv[3], argv[2], type, 0);
    }
    if (gbs_compat_status() != GBS_OK) {
        printf("status %d\n", (int)gbs_compat_status());
        return 1;
    }
    FILE *f = fopen(argv[5], "wb");
    if (!f) return 2;
    lint hdr[4] = {gs->v_size, gs->e_size, gs->offset, gs->global_v_size};
    fwrite(hdr, 8, 4, f);
    for (lint v = 0; v < gs->v_size; ++v) {
        fwrite(&gs->vet_idx[v], 8, 1, f);
        fwrite(&gs->vet_info[v].weight, 8, 1, f);
        fwrite(&gs->vet_info[v].wb, 8, 1, f);
        fwrite(&gs->vet_info[v].recip, 8, 1, f);
        fwrite(&gs->vet_info[v].vet_deg, 8, 1, f);
    }
    for (lint e = 0; e < gs->e_size; ++e) {
        fwrite(&gs->edge_idx[e], 8, 1, f);
        fwrite(&gs->edge_info[e].edge_weight, 8, 1, f);
    }
    fclose(f);
    return 0;
}
