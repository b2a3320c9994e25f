/* ss4d_vtk.c — the reference's file formats, host side: one 3D frame of a
 * 4D volume as a VTK STRUCTURED_POINTS file of unsigned bytes, and the
 * per-frame centre files.  The byte <-> double conversions run on the GPU
 * (ss4d_frame_from_bytes / ss4d_frame_to_bytes), so a frame crosses the bus
 * as one byte per voxel.
 *
 *   frame file, written (segmentation4D.c:1229-1258, segmentation4D_mpi.c:
 *   1445-1473): ten header lines, then nx*ny*nz bytes, x fastest;
 *   frame file, read (_load3dDataArrayVTK_, segmentation4D.c:1295-1324): ten
 *   lines skipped (each read like fgets with a 256-byte buffer), then the bytes;
 *   centre file (_readData_ with _readMetaData_ and _readNumberFromFile_,
 *   segmentation4D.c:1181-1205, 1262-1293): comment lines starting with '#'
 *   skipped, the first character of the next line taken with them, the rest
 *   of that line and two more lines skipped, then 7 characters ("POINTS "),
 *   the point count up to the next white space, the rest of that line, and
 *   the points as x y z; a centre is (double)(int)(x / spacing + 0.5). */
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/ss4d.h"

static ss4d_status fail(const char *msg)
{
    extern void ss4d_set_error_text_c(const char *msg);
    ss4d_set_error_text_c(msg);
    return SS4D_ERR_INVALID;
}

ss4d_status ss4d_vtk_write_frame(const char *path, int nx, int ny, int nz, const double origin[3],
                                 const double spacing[3], const uint8_t *bytes)
{
    if (!path || !origin || !spacing || !bytes || nx < 1 || ny < 1 || nz < 1)
        return fail("invalid argument to ss4d_vtk_write_frame");
    FILE *f = fopen(path, "wb");
    if (!f)
        return fail("ss4d_vtk_write_frame: the file could not be opened");
    fprintf(f, "# vtk DataFile Version 3.0\n");
    fprintf(f, "file in binary format\n");
    fprintf(f, "BINARY\n");
    fprintf(f, "DATASET STRUCTURED_POINTS\n");
    fprintf(f, "DIMENSIONS %d %d %d\n", nx, ny, nz);
    fprintf(f, "ORIGIN %f %f %f\n", origin[0], origin[1], origin[2]);
    fprintf(f, "SPACING %f %f %f\n", spacing[0], spacing[1], spacing[2]);
    fprintf(f, "POINT_DATA %lld\n", (long long)nx * ny * nz);
    fprintf(f, "SCALARS scalars unsigned_char\n");
    fprintf(f, "LOOKUP_TABLE default\n");
    const size_t n = (size_t)nx * ny * nz;
    const size_t w = fwrite(bytes, 1, n, f);
    const int bad = fclose(f) != 0 || w != n;
    return bad ? fail("ss4d_vtk_write_frame: short write") : SS4D_OK;
}

/* one header line as fgets(buf, 256, f) consumes it: up to 255 characters
 * or through the newline */
static int skip_line_256(FILE *f)
{
    for (int n = 0; n < 255; ++n) {
        const int c = getc(f);
        if (c == EOF)
            return -1;
        if (c == '\n')
            return 0;
    }
    return 0;
}

ss4d_status ss4d_vtk_read_frame(const char *path, int nx, int ny, int nz, uint8_t *bytes)
{
    if (!path || !bytes || nx < 1 || ny < 1 || nz < 1)
        return fail("invalid argument to ss4d_vtk_read_frame");
    FILE *f = fopen(path, "rb");
    if (!f)
        return fail("ss4d_vtk_read_frame: the file could not be opened");
    for (int h = 0; h < 10; ++h)
        if (skip_line_256(f) != 0) {
            fclose(f);
            return fail("ss4d_vtk_read_frame: truncated header");
        }
    const size_t n = (size_t)nx * ny * nz;
    const size_t r = fread(bytes, 1, n, f);
    fclose(f);
    /* the reference takes EOF (-1) / 255 for missing bytes; refuse instead */
    return r == n ? SS4D_OK : fail("ss4d_vtk_read_frame: fewer voxels than the volume needs");
}

ss4d_status ss4d_vtk_read_centers(const char *path, const double spacing[3], int max_points, double *cx, double *cy,
                                  double *cz, int *n_out)
{
    if (!path || !spacing || !n_out || max_points < 0 || (max_points > 0 && (!cx || !cy || !cz)))
        return fail("invalid argument to ss4d_vtk_read_centers");
    FILE *f = fopen(path, "r");
    if (!f)
        return fail("ss4d_vtk_read_centers: the file could not be opened");
    int c;
    while ((c = getc(f)) == '#') /* comment lines */
        while ((c = getc(f)) != '\n' && c != EOF)
            ;
    for (int h = 0; h < 3 && c != EOF; ++h) /* the rest of that line, then two lines */
        while ((c = getc(f)) != '\n' && c != EOF)
            ;
    char word[8] = {0};
    if (c == EOF || !fgets(word, 8, f)) {
        fclose(f);
        return fail("ss4d_vtk_read_centers: truncated header");
    }
    char num[64];
    int k = 0;
    do {
        c = getc(f);
        if (k < (int)sizeof num - 1)
            num[k++] = (char)c;
    } while (c != EOF && !isspace(c));
    num[k] = 0;
    const int points = atoi(num);
    do /* to the end of the line, reading at least one more character (as the reference) */
        c = getc(f);
    while (c != '\n' && c != EOF);
    if (points < 0 || points > max_points) {
        fclose(f);
        return fail("ss4d_vtk_read_centers: more points than the caller's arrays hold");
    }
    for (int i = 0; i < points; ++i) {
        double x, y, z;
        if (fscanf(f, "%lf", &x) != 1 || fscanf(f, "%lf", &y) != 1 || fscanf(f, "%lf", &z) != 1) {
            fclose(f);
            return fail("ss4d_vtk_read_centers: truncated point list");
        }
        cx[i] = (double)(int)(x / spacing[0] + 0.5);
        cy[i] = (double)(int)(y / spacing[1] + 0.5);
        cz[i] = (double)(int)(z / spacing[2] + 0.5);
    }
    fclose(f);
    *n_out = points;
    return SS4D_OK;
}
