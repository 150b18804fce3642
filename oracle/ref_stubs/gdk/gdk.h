/* Stand-in for <gdk/gdk.h>; see gtk/gtk.h. Test infrastructure only. */
#include <gtk/gtk.h>
