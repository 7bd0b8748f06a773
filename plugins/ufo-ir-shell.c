/*
 * ufo-ir-shell.c - the shells' core library: the shared libufoir context,
 * status -> GError mapping, and the method nodes' common requisition.
 */
#include <stdlib.h>
#include <string.h>

#include "ufo-ir-shell.h"

static ufoir_ctx *shell_ctx = NULL;
static GMutex shell_mutex;

ufoir_ctx *
ufo_ir_shell_context (GError **error)
{
    g_mutex_lock (&shell_mutex);

    if (shell_ctx == NULL) {
        const gchar *dev = g_getenv ("UFOIR_DEVICE");
        const int device = dev != NULL ? atoi (dev) : 0;
        ufoir_ctx *ctx = NULL;
        const int rc = ufoir_ctx_create (device, 0, &ctx);

        if (rc != UFOIR_OK) {
            g_set_error (error, UFO_TASK_ERROR, UFO_TASK_ERROR_SETUP,
                         "libufoir: no context on CUDA device %d (status %d): %s",
                         device, rc, ufoir_last_error (NULL));
        }
        else
            shell_ctx = ctx;
    }

    g_mutex_unlock (&shell_mutex);
    return shell_ctx;
}

gboolean
ufo_ir_shell_check (ufoir_ctx *ctx, int status, const gchar *what, GError **error)
{
    if (status == UFOIR_OK)
        return TRUE;

    g_set_error (error, UFO_TASK_ERROR, UFO_TASK_ERROR_SETUP, "%s failed (libufoir status %d): %s",
                 what, status, ctx != NULL ? ufoir_last_error (ctx) : "");
    return FALSE;
}

ufoir_projector *
ufo_ir_shell_projector (GObject *projector_node, GError **error)
{
    ufoir_projector *p = NULL;

    if (projector_node != NULL)
        p = (ufoir_projector *) g_object_get_data (projector_node, UFO_IR_SHELL_PROJECTOR_KEY);

    if (p == NULL)
        g_set_error (error, UFO_TASK_ERROR, UFO_TASK_ERROR_SETUP,
                     "No projector specified, or its setup has not run.");
    return p;
}

void
ufo_ir_shell_method_requisition (GObject *projector_node, UfoBuffer **inputs,
                                 UfoRequisition *requisition, GError **error)
{
    ufoir_projector *p = ufo_ir_shell_projector (projector_node, error);
    UfoRequisition in;
    size_t in_dims[2], out_dims[2];

    if (p == NULL)
        return;

    ufo_buffer_get_requisition (inputs[0], &in);
    in_dims[0] = in.dims[0];
    in_dims[1] = in.dims[1];

    if (!ufo_ir_shell_check (NULL, ufoir_projector_get_requisition (p, in_dims, out_dims),
                             "projector requisition", error))
        return;

    requisition->n_dims = 2;
    requisition->dims[0] = out_dims[0];
    requisition->dims[1] = out_dims[1];
}

int
ufo_ir_shell_norm_mode (const gchar *name)
{
    if (name != NULL && g_ascii_strcasecmp (name, "compat") == 0)
        return UFOIR_NORM_COMPAT;
    return UFOIR_NORM_FP64;
}
