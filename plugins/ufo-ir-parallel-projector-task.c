/*
 * ufo-ir-parallel-projector-task.c - the "parallel-projector" node of package
 * "ir" over libufoir.
 *
 * Replaces src/tasks/ufo-ir-parallel-projector-task.c with its properties
 * (model :123-128, angles_num :132-137), those of the projector and
 * state-dependent bases it inherits (src/core/ufo-ir-projector-task.c:68-93:
 * axis_position, step, relaxation, correction_scale, with their ranges;
 * src/core/ufo-ir-state-dependent-task.c:75-80: is_forward), its
 * requisition (:306-347) and its process (state-dependent :195-212: zero the
 * output, then forward or backward projection). Method nodes reach the
 * libufoir projector through the object's "ufoir-projector" data.
 */
#include <string.h>

#include "ufo-ir-shell.h"

typedef struct {
    UfoTaskNode parent_instance;
    ufoir_projector_params prm;
    ufoir_projector *proj;
} UfoIrParallelProjectorTask;

typedef struct {
    UfoTaskNodeClass parent_class;
} UfoIrParallelProjectorTaskClass;

static void ufo_task_interface_init (UfoTaskIface *iface);

G_DEFINE_TYPE_WITH_CODE (UfoIrParallelProjectorTask, ufo_ir_parallel_projector_task, UFO_TYPE_TASK_NODE,
                         G_IMPLEMENT_INTERFACE (UFO_TYPE_TASK, ufo_task_interface_init))

#define SELF(obj) ((UfoIrParallelProjectorTask *) (obj))

enum {
    PROP_0,
    PROP_MODEL,
    PROP_ANGLES_NUM,
    PROP_IS_FORWARD,
    PROP_AXIS_POSITION,
    PROP_STEP,
    PROP_RELAXATION,
    PROP_CORRECTION_SCALE,
    N_PROPERTIES
};

static GParamSpec *properties[N_PROPERTIES] = { NULL, };

UfoNode *
ufo_ir_parallel_projector_task_new (void)
{
    return UFO_NODE (g_object_new (ufo_ir_parallel_projector_task_get_type (), NULL));
}

/* pushes the node's properties into the libufoir projector, if it exists */
static void
sync_params (UfoIrParallelProjectorTask *self)
{
    if (self->proj != NULL)
        ufoir_projector_set_params (self->proj, &self->prm);
}

/* the libufoir projector may have changed relaxation / correction_scale
 * (methods leave them where the reference leaves them) */
static void
pull_params (UfoIrParallelProjectorTask *self)
{
    if (self->proj != NULL)
        ufoir_projector_get_params (self->proj, &self->prm);
}

static void
ufo_ir_parallel_projector_task_set_property (GObject *object, guint property_id, const GValue *value,
                                             GParamSpec *pspec)
{
    UfoIrParallelProjectorTask *self = SELF (object);

    pull_params (self);
    switch (property_id) {
        case PROP_MODEL:
            g_strlcpy (self->prm.model, g_value_get_string (value) ? g_value_get_string (value) : "joseph",
                       sizeof (self->prm.model));
            break;
        case PROP_ANGLES_NUM:
            self->prm.angles_num = g_value_get_uint (value);
            break;
        case PROP_IS_FORWARD:
            self->prm.is_forward = g_value_get_boolean (value);
            break;
        case PROP_AXIS_POSITION:
            self->prm.axis_position = g_value_get_float (value);
            break;
        case PROP_STEP:
            self->prm.step = g_value_get_float (value);
            break;
        case PROP_RELAXATION:
            self->prm.relaxation = g_value_get_float (value);
            break;
        case PROP_CORRECTION_SCALE:
            self->prm.correction_scale = g_value_get_float (value);
            break;
        default:
            G_OBJECT_WARN_INVALID_PROPERTY_ID (object, property_id, pspec);
            return;
    }
    sync_params (self);
}

static void
ufo_ir_parallel_projector_task_get_property (GObject *object, guint property_id, GValue *value,
                                             GParamSpec *pspec)
{
    UfoIrParallelProjectorTask *self = SELF (object);

    pull_params (self);
    switch (property_id) {
        case PROP_MODEL:
            g_value_set_string (value, self->prm.model);
            break;
        case PROP_ANGLES_NUM:
            g_value_set_uint (value, self->prm.angles_num);
            break;
        case PROP_IS_FORWARD:
            g_value_set_boolean (value, self->prm.is_forward);
            break;
        case PROP_AXIS_POSITION:
            g_value_set_float (value, self->prm.axis_position);
            break;
        case PROP_STEP:
            g_value_set_float (value, self->prm.step);
            break;
        case PROP_RELAXATION:
            g_value_set_float (value, self->prm.relaxation);
            break;
        case PROP_CORRECTION_SCALE:
            g_value_set_float (value, self->prm.correction_scale);
            break;
        default:
            G_OBJECT_WARN_INVALID_PROPERTY_ID (object, property_id, pspec);
            break;
    }
}

static void
ufo_ir_parallel_projector_task_finalize (GObject *object)
{
    UfoIrParallelProjectorTask *self = SELF (object);

    if (self->proj != NULL) {
        ufoir_projector_destroy (self->proj);
        self->proj = NULL;
    }
    G_OBJECT_CLASS (ufo_ir_parallel_projector_task_parent_class)->finalize (object);
}

/* UfoTask setup: the libufoir projector on the shared context (the
 * reference loads projector-parallel-<model>.cl here, :360-388) */
static void
ufo_ir_parallel_projector_task_setup (UfoTask *task, UfoResources *resources, GError **error)
{
    UfoIrParallelProjectorTask *self = SELF (task);
    ufoir_ctx *ctx;

    if (self->proj != NULL)
        return;
    ctx = ufo_ir_shell_context (error);
    if (ctx == NULL)
        return;
    if (!ufo_ir_shell_check (ctx, ufoir_projector_create (ctx, &self->prm, &self->proj),
                             "parallel-projector setup", error))
        return;
    g_object_set_data (G_OBJECT (self), UFO_IR_SHELL_PROJECTOR_KEY, self->proj);
}

static void
ufo_ir_parallel_projector_task_get_requisition (UfoTask *task, UfoBuffer **inputs, UfoRequisition *requisition,
                                                GError **error)
{
    UfoIrParallelProjectorTask *self = SELF (task);
    UfoRequisition in;
    size_t in_dims[2], out_dims[2];

    if (self->proj == NULL) {
        g_set_error (error, UFO_TASK_ERROR, UFO_TASK_ERROR_SETUP, "parallel-projector: setup has not run");
        return;
    }
    ufo_buffer_get_requisition (inputs[0], &in);
    in_dims[0] = in.dims[0];
    in_dims[1] = in.dims[1];
    if (!ufo_ir_shell_check (NULL, ufoir_projector_get_requisition (self->proj, in_dims, out_dims),
                             "parallel-projector requisition", error))
        return;
    requisition->n_dims = 2;
    requisition->dims[0] = out_dims[0];
    requisition->dims[1] = out_dims[1];
}

static guint
ufo_ir_parallel_projector_task_get_num_inputs (UfoTask *task)
{
    return 1;
}

static guint
ufo_ir_parallel_projector_task_get_num_dimensions (UfoTask *task, guint input)
{
    g_return_val_if_fail (input == 0, 0);
    return 2;
}

/* A processor whose data arrive as host arrays; the GPU work is libufoir's. */
static UfoTaskMode
ufo_ir_parallel_projector_task_get_mode (UfoTask *task)
{
    return UFO_TASK_MODE_PROCESSOR | UFO_TASK_MODE_CPU;
}

static gboolean
ufo_ir_parallel_projector_task_process (UfoTask *task, UfoBuffer **inputs, UfoBuffer *output,
                                        UfoRequisition *requisition)
{
    UfoIrParallelProjectorTask *self = SELF (task);
    UfoRequisition in;
    size_t in_dims[2];
    int rc;

    ufo_buffer_get_requisition (inputs[0], &in);
    in_dims[0] = in.dims[0];
    in_dims[1] = in.dims[1];
    rc = ufoir_projector_process (self->proj, ufo_buffer_get_host_array (inputs[0], NULL), in_dims,
                                  ufo_buffer_get_host_array (output, NULL), 1);
    if (rc != UFOIR_OK)
        g_warning ("parallel-projector: process failed (libufoir status %d)", rc);
    return TRUE;
}

static void
ufo_task_interface_init (UfoTaskIface *iface)
{
    iface->setup = ufo_ir_parallel_projector_task_setup;
    iface->get_requisition = ufo_ir_parallel_projector_task_get_requisition;
    iface->get_num_inputs = ufo_ir_parallel_projector_task_get_num_inputs;
    iface->get_num_dimensions = ufo_ir_parallel_projector_task_get_num_dimensions;
    iface->get_mode = ufo_ir_parallel_projector_task_get_mode;
    iface->process = ufo_ir_parallel_projector_task_process;
}

static void
ufo_ir_parallel_projector_task_class_init (UfoIrParallelProjectorTaskClass *klass)
{
    GObjectClass *oclass = G_OBJECT_CLASS (klass);

    oclass->set_property = ufo_ir_parallel_projector_task_set_property;
    oclass->get_property = ufo_ir_parallel_projector_task_get_property;
    oclass->finalize = ufo_ir_parallel_projector_task_finalize;

    properties[PROP_MODEL] =
        g_param_spec_string ("model", "The name of the projection model.", "The name of the projection model.",
                             "joseph", G_PARAM_READWRITE);
    properties[PROP_ANGLES_NUM] =
        g_param_spec_uint ("angles_num", "Amount of angles for forward projection",
                           "Amount of angles for forward projection (0: from the input)", 0, G_MAXUINT, 0,
                           G_PARAM_READWRITE);
    properties[PROP_IS_FORWARD] =
        g_param_spec_boolean ("is_forward", "Forward (TRUE) or backward (FALSE) projection",
                              "Forward (TRUE) or backward (FALSE) projection", TRUE, G_PARAM_READWRITE);
    properties[PROP_AXIS_POSITION] =
        g_param_spec_float ("axis_position", "Rotation axis position", "Rotation axis position (-1: n_dets / 2)",
                            -1.0f, G_MAXFLOAT, -1.0f, G_PARAM_READWRITE);
    properties[PROP_STEP] =
        g_param_spec_float ("step", "Angle step in radians", "Angle step in radians", 0.0f, G_MAXFLOAT, 0.0f,
                            G_PARAM_READWRITE);
    properties[PROP_RELAXATION] =
        g_param_spec_float ("relaxation", "Projection relaxation parameter", "Projection relaxation parameter",
                            G_MINFLOAT, G_MAXFLOAT, 1.0f, G_PARAM_READWRITE);
    properties[PROP_CORRECTION_SCALE] =
        g_param_spec_float ("correction_scale", "FP correction scale", "FP correction scale", G_MINFLOAT,
                            G_MAXFLOAT, 1.0f, G_PARAM_READWRITE);

    for (guint i = PROP_0 + 1; i < N_PROPERTIES; i++)
        g_object_class_install_property (oclass, i, properties[i]);
}

static void
ufo_ir_parallel_projector_task_init (UfoIrParallelProjectorTask *self)
{
    ufoir_projector_params_init (&self->prm);
    self->proj = NULL;
}
