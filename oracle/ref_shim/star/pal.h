/* Declarations of the PAL (Starlink Positional Astronomy Library) routines that the reference's
 * src/pacer_geometry.h names.  PAL is not available here; the golden driver calls only the
 * geometry routines that need none of them (precXYZ, CalcUVW), so nothing here is defined. */
#ifndef GB300_SHIM_STAR_PAL_H
#define GB300_SHIM_STAR_PAL_H
void palCaldj(int iy, int im, int id, double *djm, int *j);
void palDcc2s(double v[3], double *a, double *b);
void palDcs2c(double a, double b, double v[3]);
void palDmxv(double dm[3][3], double va[3], double vb[3]);
double palDranrm(double angle);
double palDvdv(double va[3], double vb[3]);
void palDvn(double v[3], double uv[3], double *vm);
double palGmst(double ut1);
void palMap(double rm, double dm, double pr, double pd, double px, double rv, double eq, double date,
            double *ra, double *da);
void palMappa(double eq, double date, double amprms[21]);
void palPrenut(double epoch, double date, double rmatpn[3][3]);
#endif
