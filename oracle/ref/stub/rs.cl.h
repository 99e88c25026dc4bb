/* Empty stand-in for the rs.cl.h that rs.c includes (rs.c:14): the file is
 * not part of the reference tree and rs.c uses nothing from it (the kernel
 * source is read from rs.cl at run time, rs.c:1083-1110). */
