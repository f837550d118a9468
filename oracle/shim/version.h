/* Empty stand-in for the install-time generated header that the reference's
 * stdinc.h includes; load.c / grav.c / ran3.c need nothing from it. */
