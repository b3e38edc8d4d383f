/*
 * gpubackend — drop-in replacement for CircuitSimulator's libcirc/mpibackend.
 *
 * Same command line and stdin protocol as the reference master
 * (libcirc/probability.c:44-68): with one argument it is the input file, or
 * "stdin"; with none, a file name is read from stdin.  libcirc/probability.py
 * runs it with config["cpath"] = path of this executable and
 * config["mpirun"] = "" (one process drives the whole GPU).
 *
 * "gpubackend serve" keeps one process for a stream of back-to-back protocol
 * inputs and answers each with one line (csim_backend_serve).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/csim.h"

int main(int argc, char *argv[]) {
    char file[256] = "";
    if (argc == 2 && strcmp(argv[1], "serve") == 0) {  /* one process, a stream of queries */
        const char *dev = getenv("CSIM_DEVICE");
        return csim_backend_serve(stdin, stdout, dev ? atoi(dev) : 0) == CSIM_OK ? 0 : 1;
    }
    printf("C backend print mode is on.\n");
    if (argc == 1) {
        if (scanf("%255s", file) != 1) file[0] = '\0';
    } else {
        strncpy(file, argv[1], sizeof(file) - 1);
    }
    FILE *stream;
    if (strlen(file) == 0 || strcmp(file, "stdin") == 0) {
        printf("Reading arguments from stdin\n");
        stream = stdin;
    } else {
        printf("Reading arguments from file: %s\n", file);
        stream = fopen(file, "r");
        if (stream == NULL) {
            printf("Error reading file.\n");
            return 0;
        }
    }
    const char *dev = getenv("CSIM_DEVICE");
    int rc = csim_backend_run(stream, stdout, dev ? atoi(dev) : 0);
    if (stream != stdin) fclose(stream);
    return rc == CSIM_OK ? 0 : 1;
}
