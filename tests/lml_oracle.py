"""The oracle's LML for the FitzHugh--Nagumo configuration, differentiated by
PyTorch autograd with respect to the parameters and the initial values
(``oracle.lml``, with the configuration's observation noise as default)."""

from oracle import lml as _lml
from tests import lml_problem


def lml_value_and_grads(theta, y0, data, dt, num_steps, save_every, average_pdfs=False, field="fitzhugh_nagumo",
                        num_derivatives=3, std=lml_problem.STD):
    """Returns (lml, d lml / d theta, d lml / d y0) as (float, ndarray, ndarray)."""
    return _lml.lml_value_and_grads(theta, y0, data, dt, num_steps, save_every, std, average_pdfs=average_pdfs,
                                    field=field, num_derivatives=num_derivatives)
