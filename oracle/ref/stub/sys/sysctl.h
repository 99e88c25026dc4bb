/* Empty stand-in for <sys/sysctl.h>, which glibc 2.32 and later no longer ship.
 * The reference includes it (rs_types.h:24) but the modules built here use
 * nothing from it. */
