"""FP32 reference of the warm-start MLP (4 -> 64 -> 64 -> 1, tanh-form GELU) for the
kernel tests: the parameter layout of bbg_mlp_get_params, a BF16-emulating forward for
the tensor-core inference kernel and a torch autograd forward for the training kernel."""
import numpy as np

N_IN, N_HID = 4, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_IN * N_HID
OFF_W2 = OFF_B1 + N_HID
OFF_B2 = OFF_W2 + N_HID * N_HID
OFF_W3 = OFF_B2 + N_HID
OFF_B3 = OFF_W3 + N_HID
N_PARAMS = OFF_B3 + 1
GELU_C = np.sqrt(2.0 / np.pi)
GELU_A = 0.044715


def unpack(theta):
    t = np.asarray(theta, np.float32)
    return (t[OFF_W1:OFF_B1].reshape(N_IN, N_HID), t[OFF_B1:OFF_W2], t[OFF_W2:OFF_B2].reshape(N_HID, N_HID),
            t[OFF_B2:OFF_W3], t[OFF_W3:OFF_B3], t[OFF_B3])


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + GELU_A * x ** 3)))


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


GELU_A_FOLD = GELU_A / (GELU_C * GELU_C)


def gelu_folded_bf16(y):
    """The inference kernel's hidden activation h = y (1 + tanh(y + a' y^3)), a' = a / c^2,
    of y = c x, in BF16 arithmetic: rounding after every operation as its paired BF16
    instructions do (a fused multiply-add rounds once).  GELU(x) = (0.5 / c) h."""
    a = bf16(np.float32(GELU_A_FOLD))
    y = bf16(y)
    ay2 = bf16(bf16(y * y) * a)
    u = bf16((ay2.astype(np.float64) * y + y).astype(np.float32))
    t = bf16(np.tanh(u.astype(np.float64)).astype(np.float32))
    return bf16((y.astype(np.float64) * t + y).astype(np.float32))


def forward_bf16(theta, x):
    """What the inference kernel computes: GELU's constants folded into the weights (layer 1
    holds c W1, c b1; layer 2 0.5 W2, c b2; layer 3 (0.5 / c) w3), BF16 inputs and weights,
    FP32 accumulation, the BF16 activation of both hidden layers, BF16 w3 and an FP32
    output dot product."""
    w1, b1, w2, b2, w3, b3 = unpack(theta)
    c = np.float32(GELU_C)
    x = bf16(np.asarray(x, np.float32)).astype(np.float64)
    y1 = (x @ bf16(c * w1).astype(np.float64) + bf16(c * b1).astype(np.float64)).astype(np.float32)
    h1 = gelu_folded_bf16(y1).astype(np.float64)
    y2 = (h1 @ bf16(np.float32(0.5) * w2).astype(np.float64) + (c * b2).astype(np.float64)).astype(np.float32)
    h2 = gelu_folded_bf16(y2).astype(np.float64)
    return (h2 @ bf16(np.float32(0.5) / c * w3).astype(np.float64) + float(b3)).astype(np.float32)


def loss_and_grad(theta, x, t, expectile=0.5):
    """Mean (expectile-weighted) squared error and its gradient in FP32 (torch autograd,
    CPU): errors above the target weigh 2 (1 - tau), below 2 tau."""
    import torch
    th = torch.tensor(np.asarray(theta, np.float32), requires_grad=True)
    w1 = th[OFF_W1:OFF_B1].reshape(N_IN, N_HID)
    b1 = th[OFF_B1:OFF_W2]
    w2 = th[OFF_W2:OFF_B2].reshape(N_HID, N_HID)
    b2 = th[OFF_B2:OFF_W3]
    w3 = th[OFF_W3:OFF_B3]
    b3 = th[OFF_B3]

    def g(z):
        return 0.5 * z * (1.0 + torch.tanh(GELU_C * (z + GELU_A * z ** 3)))

    xt = torch.tensor(np.asarray(x, np.float32))
    y = g(g(xt @ w1 + b1) @ w2 + b2) @ w3 + b3
    err = y - torch.tensor(np.asarray(t, np.float32))
    w = torch.where(err > 0, 2.0 * (1.0 - expectile), 2.0 * expectile)
    loss = (w.detach() * err ** 2).mean()
    loss.backward()
    return float(loss.detach()), th.grad.numpy().copy()
