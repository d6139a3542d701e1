"""acc/components/sources/STS_source.py: the STS moderator source, the SNS
source's energy and time draws on the STS moderator's geometry.  It is the
SNS source opcode with the STS flags (MCV_OP_SNS_SOURCE, ip[7]); the class
lives beside SNS_source."""

from .SNS_source import STS_source  # noqa: F401

category = 'sources'
