/* Empty autoconf config.h so that mark5access 1.4.3 compiles without running
 * its configure script (the sources include "config.h" unconditionally). */
