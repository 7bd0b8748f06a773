/*
 * ufo-ir-sirt-task.c - the "sirt" node of package "ir" over libufoir.
 *
 * Replaces src/tasks/ufo-ir-sirt-task.c: property relaxation_factor
 * [0, 1] default 0.25 (:73-77) on top of the method base; process
 * (:164-222) is ufoir_sirt_process on the node's one sinogram.
 */
#include "ufo-ir-method-shell.h"

typedef struct {
    UfoIrMethodShell base;
    gfloat relaxation_factor;
} UfoIrSirtTask;

typedef struct {
    UfoTaskNodeClass parent_class;
} UfoIrSirtTaskClass;

static void ufo_task_interface_init (UfoTaskIface *iface);

G_DEFINE_TYPE_WITH_CODE (UfoIrSirtTask, ufo_ir_sirt_task, UFO_TYPE_TASK_NODE,
                         G_IMPLEMENT_INTERFACE (UFO_TYPE_TASK, ufo_task_interface_init))

#define SELF(obj) ((UfoIrSirtTask *) (obj))

enum { PROP_RELAXATION_FACTOR = UFO_IR_METHOD_PROP_FIRST_OWN };

UfoNode *
ufo_ir_sirt_task_new (void)
{
    return UFO_NODE (g_object_new (ufo_ir_sirt_task_get_type (), NULL));
}

static void
ufo_ir_sirt_task_set_property (GObject *object, guint property_id, const GValue *value, GParamSpec *pspec)
{
    UfoIrSirtTask *self = SELF (object);

    if (ufo_ir_method_shell_set (&self->base, property_id, value))
        return;
    if (property_id == PROP_RELAXATION_FACTOR)
        self->relaxation_factor = g_value_get_float (value);
    else
        G_OBJECT_WARN_INVALID_PROPERTY_ID (object, property_id, pspec);
}

static void
ufo_ir_sirt_task_get_property (GObject *object, guint property_id, GValue *value, GParamSpec *pspec)
{
    UfoIrSirtTask *self = SELF (object);

    if (ufo_ir_method_shell_get (&self->base, property_id, value))
        return;
    if (property_id == PROP_RELAXATION_FACTOR)
        g_value_set_float (value, self->relaxation_factor);
    else
        G_OBJECT_WARN_INVALID_PROPERTY_ID (object, property_id, pspec);
}

static void
ufo_ir_sirt_task_dispose (GObject *object)
{
    ufo_ir_method_shell_dispose (&SELF (object)->base);
    G_OBJECT_CLASS (ufo_ir_sirt_task_parent_class)->dispose (object);
}

static void
ufo_ir_sirt_task_setup (UfoTask *task, UfoResources *resources, GError **error)
{
    ufo_ir_method_shell_setup (&SELF (task)->base, resources, error);
}

static void
ufo_ir_sirt_task_get_requisition (UfoTask *task, UfoBuffer **inputs, UfoRequisition *requisition, GError **error)
{
    ufo_ir_shell_method_requisition (SELF (task)->base.projector, inputs, requisition, error);
}

static guint
ufo_ir_sirt_task_get_num_inputs (UfoTask *task)
{
    return 1;
}

static guint
ufo_ir_sirt_task_get_num_dimensions (UfoTask *task, guint input)
{
    g_return_val_if_fail (input == 0, 0);
    return 2;
}

static UfoTaskMode
ufo_ir_sirt_task_get_mode (UfoTask *task)
{
    return UFO_TASK_MODE_PROCESSOR | UFO_TASK_MODE_CPU;
}

static gboolean
ufo_ir_sirt_task_process (UfoTask *task, UfoBuffer **inputs, UfoBuffer *output, UfoRequisition *requisition)
{
    UfoIrSirtTask *self = SELF (task);
    ufoir_projector *proj = ufo_ir_shell_projector (self->base.projector, NULL);
    ufoir_sirt_params prm;
    size_t dims[2];

    if (proj == NULL)
        return ufo_ir_method_shell_done ("sirt", UFOIR_ERR_STATE);
    ufoir_sirt_params_init (&prm);
    prm.num_iterations = self->base.num_iterations;
    prm.relaxation_factor = self->relaxation_factor;
    ufo_ir_method_shell_dims (inputs[0], dims);
    return ufo_ir_method_shell_done ("sirt",
        ufoir_sirt_process (proj, &prm, ufo_buffer_get_host_array (inputs[0], NULL), dims,
                            ufo_buffer_get_host_array (output, NULL), 1));
}

static void
ufo_task_interface_init (UfoTaskIface *iface)
{
    iface->setup = ufo_ir_sirt_task_setup;
    iface->get_requisition = ufo_ir_sirt_task_get_requisition;
    iface->get_num_inputs = ufo_ir_sirt_task_get_num_inputs;
    iface->get_num_dimensions = ufo_ir_sirt_task_get_num_dimensions;
    iface->get_mode = ufo_ir_sirt_task_get_mode;
    iface->process = ufo_ir_sirt_task_process;
}

static void
ufo_ir_sirt_task_class_init (UfoIrSirtTaskClass *klass)
{
    GObjectClass *oclass = G_OBJECT_CLASS (klass);

    oclass->set_property = ufo_ir_sirt_task_set_property;
    oclass->get_property = ufo_ir_sirt_task_get_property;
    oclass->dispose = ufo_ir_sirt_task_dispose;
    ufo_ir_method_shell_install (oclass);
    g_object_class_install_property (oclass, PROP_RELAXATION_FACTOR,
        g_param_spec_float ("relaxation_factor", "relaxation_factor", "Relaxation factor", 0.0f, 1.0f, 0.25f,
                            G_PARAM_READWRITE));
}

static void
ufo_ir_sirt_task_init (UfoIrSirtTask *self)
{
    ufo_ir_method_shell_init (&self->base);
    self->relaxation_factor = 0.25f;
}
