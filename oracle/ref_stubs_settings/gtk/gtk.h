/* Stand-in for <gtk/gtk.h> used to compile the reference's settings reader
 * (src/settings.cpp) for the oracle's pinning harness: the post-processing stub plus
 * GLib's locale-independent number conversions and the message-dialog calls on the
 * reader's GUI-only path (never reached: the harness runs with noGUI set).
 * g_ascii_strtod behaves as strtod in the "C" numeric locale, which the harness keeps.
 * Test infrastructure only. */
#ifndef MBGB_REF_STUB_GTK_SETTINGS_H
#define MBGB_REF_STUB_GTK_SETTINGS_H
#include <stdio.h>
#include <stdlib.h>
#include "../../ref_stubs_post/gtk/gtk.h"
#define G_ASCII_DTOSTR_BUF_SIZE 39
static inline double g_ascii_strtod(const char *s, char **end) { return strtod(s, end); }
static inline char *g_ascii_dtostr(char *buf, int len, double d) {
  snprintf(buf, (size_t)len, "%.17g", d);
  return buf;
}
#define GTK_WINDOW(x) (x)
#define GTK_DIALOG(x) (x)
#define GTK_DIALOG_MODAL 0
#define GTK_MESSAGE_WARNING 0
#define GTK_MESSAGE_ERROR 0
#define GTK_BUTTONS_OK 0
#define GTK_BUTTONS_CANCEL 0
static inline GtkWidget *gtk_message_dialog_new(void *, int, int, int, const char *, ...) { return 0; }
static inline int gtk_dialog_run(void *) { return 0; }
static inline void gtk_widget_destroy(void *) {}
#endif
