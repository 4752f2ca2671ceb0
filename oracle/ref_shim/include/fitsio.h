/* Empty stand-in: the reference includes this HEALPix/cfitsio header but the
 * compiled files use nothing from it. */
