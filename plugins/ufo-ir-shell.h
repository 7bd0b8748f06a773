/*
 * ufo-ir-shell.h - shared parts of the ufo-core plugin shells over libufoir.
 *
 * The shells are the GObject plugins ufo-core loads for the "ir" package
 * (libufo<name>.so, exporting ufo_ir_<name>_task_new; reference:
 * src/CMakeLists.txt:39-59, src/tasks/ufo-ir-sart-task.c:146-150). They keep
 * the reference plugins' node names, property names, types, ranges and
 * defaults, and run the work through the C ABI of include/ufoir.h on the
 * GPU: data reach it as the UfoBuffers' host arrays (ufo-core's buffers are
 * OpenCL objects, which CUDA cannot map, so the host array is the hand-over
 * point), and the results go back the same way.
 *
 * This header and ufo-ir-shell.c form the shells' core library (libufo-ir,
 * the name of the reference's core library, src/CMakeLists.txt:34).
 */
#ifndef UFO_IR_SHELL_H
#define UFO_IR_SHELL_H

#include <ufo/ufo.h>

#include "ufoir.h"

G_BEGIN_DECLS

/* The libufoir context the shells share in this process: one per CUDA
 * device, created on first use on the device named by $UFOIR_DEVICE (default
 * 0) and kept until exit. NULL (and *error set) if it cannot be made. */
ufoir_ctx *ufo_ir_shell_context (GError **error);

/* Sets *error from a libufoir status and the context's last message;
 * returns TRUE when status is UFOIR_OK. */
gboolean ufo_ir_shell_check (ufoir_ctx *ctx, int status, const gchar *what, GError **error);

/* The libufoir projector of a "parallel-projector" node (set up by its
 * UfoTask setup), or NULL with *error set. */
ufoir_projector *ufo_ir_shell_projector (GObject *projector_node, GError **error);

/* Name of the GObject data key under which the projector node keeps its
 * ufoir_projector handle. */
#define UFO_IR_SHELL_PROJECTOR_KEY "ufoir-projector"

/* Requisition of a method node: the projector node's, as the reference's
 * method base delegates it (src/core/ufo-ir-method-task.c:221-233). */
void ufo_ir_shell_method_requisition (GObject *projector_node, UfoBuffer **inputs,
                                      UfoRequisition *requisition, GError **error);

/* "norm-mode" property values ("compat" | "fp64"), an extension with no
 * counterpart in the reference (its norms are float sequential sums). */
int ufo_ir_shell_norm_mode (const gchar *name);

G_END_DECLS

#endif
