// Stand-in for cfitsio's header: only the opaque type the reference's headers name.
#ifndef BGI_SHIM_FITSIO_H
#define BGI_SHIM_FITSIO_H
typedef struct bgi_shim_fitsfile fitsfile;
#endif
