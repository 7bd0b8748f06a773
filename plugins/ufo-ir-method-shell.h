/*
 * ufo-ir-method-shell.h - the parts every method node shares, after the
 * reference's method base (src/core/ufo-ir-method-task.c): the
 * "num-iterations" and "projector" properties (:75-86), setup of the
 * projector (:208-219), one input of two dimensions, and the projector's
 * requisition (:221-233).
 *
 * A method's instance struct starts with UfoIrMethodShell.
 */
#ifndef UFO_IR_METHOD_SHELL_H
#define UFO_IR_METHOD_SHELL_H

#include "ufo-ir-shell.h"

G_BEGIN_DECLS

typedef struct {
    UfoTaskNode parent_instance;
    guint num_iterations;
    GObject *projector;          /* a "parallel-projector" node, held with a reference */
} UfoIrMethodShell;

enum { UFO_IR_METHOD_PROP_ITERATIONS = 1, UFO_IR_METHOD_PROP_PROJECTOR = 2, UFO_IR_METHOD_PROP_FIRST_OWN = 3 };

static inline void
ufo_ir_method_shell_install (GObjectClass *oclass)
{
    g_object_class_install_property (oclass, UFO_IR_METHOD_PROP_ITERATIONS,
        g_param_spec_uint ("num-iterations", "Number of iterations of method", "Number of iterations of method",
                           1, G_MAXUINT, 10, G_PARAM_READWRITE));
    g_object_class_install_property (oclass, UFO_IR_METHOD_PROP_PROJECTOR,
        g_param_spec_object ("projector", "Current projector", "Current projector", G_TYPE_OBJECT,
                             G_PARAM_READWRITE));
}

static inline void
ufo_ir_method_shell_init (UfoIrMethodShell *m)
{
    m->num_iterations = 10;
    m->projector = NULL;
}

/* TRUE if property_id was one of the base's */
static inline gboolean
ufo_ir_method_shell_set (UfoIrMethodShell *m, guint property_id, const GValue *value)
{
    if (property_id == UFO_IR_METHOD_PROP_ITERATIONS) {
        m->num_iterations = g_value_get_uint (value);
        return TRUE;
    }
    if (property_id == UFO_IR_METHOD_PROP_PROJECTOR) {
        GObject *p = g_value_get_object (value);
        if (m->projector != NULL)
            g_object_unref (m->projector);
        m->projector = p != NULL ? g_object_ref_sink (p) : NULL;
        return TRUE;
    }
    return FALSE;
}

static inline gboolean
ufo_ir_method_shell_get (UfoIrMethodShell *m, guint property_id, GValue *value)
{
    if (property_id == UFO_IR_METHOD_PROP_ITERATIONS) {
        g_value_set_uint (value, m->num_iterations);
        return TRUE;
    }
    if (property_id == UFO_IR_METHOD_PROP_PROJECTOR) {
        g_value_set_object (value, m->projector);
        return TRUE;
    }
    return FALSE;
}

static inline void
ufo_ir_method_shell_dispose (UfoIrMethodShell *m)
{
    if (m->projector != NULL) {
        g_object_unref (m->projector);
        m->projector = NULL;
    }
}

static inline void
ufo_ir_method_shell_setup (UfoIrMethodShell *m, UfoResources *resources, GError **error)
{
    if (m->projector == NULL)
        g_set_error (error, UFO_TASK_ERROR, UFO_TASK_ERROR_SETUP, "No projector specified.");
    else
        ufo_task_setup (UFO_TASK (m->projector), resources, error);
}

/* The sinogram's dims as the C ABI takes them: {n_dets, n_angles}. */
static inline void
ufo_ir_method_shell_dims (UfoBuffer *sino, size_t dims[2])
{
    UfoRequisition req;
    ufo_buffer_get_requisition (sino, &req);
    dims[0] = req.dims[0];
    dims[1] = req.dims[1];
}

/* process() result: the reference's process returns TRUE and logs errors. */
static inline gboolean
ufo_ir_method_shell_done (const gchar *name, int rc)
{
    if (rc != UFOIR_OK)
        g_warning ("%s: process failed (libufoir status %d)", name, rc);
    return TRUE;
}

G_END_DECLS

#endif
