// Command-line driver with the reference's argument forms (main, sdpa_main.cpp:501-677):
//   sdpa_gmp_gb300 (-ds data.dat-s | -dd data.dat) -o out.result [-p param.sdpa] [-pt 0|1|2]
//                  [-is init | -id init]
//   sdpa_gmp_gb300 data out.result [param.sdpa]   (a data name ending in "-s" is sparse)
// It solves on GPU 0 (SDPG_DEVICE selects another) through the library's C ABI and writes
// the reference's result-file layout.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "sdpg.h"

static int usage(const char *prog) {
    fprintf(stderr,
            "usage: %s (-ds data.dat-s | -dd data.dat) -o out.result [-p param.sdpa] [-pt 0|1|2] [-is|-id init]\n"
            "       %s data.dat-s out.result [param.sdpa]\n",
            prog, prog);
    return 1;
}

int main(int argc, char **argv) {
    setbuf(stdout, NULL);
    const time_t now = time(NULL);
    printf("SDPA-GMP start at    %s", ctime(&now));
    if (argc < 3) return usage(argv[0]);
    const char *data = NULL, *out = NULL, *par = NULL, *init = NULL;
    int preset = -1, init_sparse = 0, dense = 0;
    if (argv[1][0] == '-') {
        for (int i = 1; i < argc; ++i) {
            const char *a = argv[i];
            const int has = i + 1 < argc;
            if ((!strcmp(a, "-ds") || !strcmp(a, "-dd")) && has) {
                dense = !strcmp(a, "-dd");
                data = argv[++i];
            } else if (!strcmp(a, "-o") && has) {
                out = argv[++i];
            } else if (!strcmp(a, "-p") && has) {
                par = argv[++i];
                preset = -1;
            } else if (!strcmp(a, "-pt") && has) {
                preset = atoi(argv[++i]);
                if (preset < 0 || preset > 2) preset = 0;
                par = NULL;
            } else if ((!strcmp(a, "-is") || !strcmp(a, "-id")) && has) {
                init_sparse = !strcmp(a, "-is");
                init = argv[++i];
            } else if (!strcmp(a, "-k") && has) {
                ++i;  // the F1/F2/F3 cost factor stays at its default of 1.2
            } else {
                return usage(argv[0]);
            }
        }
    } else {
        data = argv[1];
        out = argv[2];
        if (argc > 3) par = argv[3];
        const size_t len = strlen(data);
        dense = !(len >= 2 && data[len - 1] == 's' && data[len - 2] == '-');
    }
    if (!data || !out) return usage(argv[0]);
    const char *dev_env = getenv("SDPG_DEVICE");
    const int device = dev_env ? atoi(dev_env) : 0;
    double info[12];
    int rc;
    if (preset >= 0) {
        sdpg_param prm;
        if (sdpg_param_default(&prm, preset) != SDPG_OK) {
            fprintf(stderr, "%s\n", sdpg_last_error());
            return 1;
        }
        rc = sdpg_solve_file_ex(data, dense, &prm, NULL, init, init_sparse, out, device, 1, info);
    } else {
        rc = sdpg_solve_file_ex(data, dense, NULL, par, init, init_sparse, out, device, 1, info);
    }
    if (rc < 0) {
        fprintf(stderr, "%s: %s\n", argv[0], sdpg_last_error());
        return 1;
    }
    printf("phase.value = %d, iterations = %d, objValPrimal = %.16e, objValDual = %.16e\n", (int)info[0],
           (int)info[1], info[2], info[3]);
    return 0;
}
