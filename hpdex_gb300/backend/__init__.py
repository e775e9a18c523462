from .mannwhitneyu_ import group_mean, mannwhitneyu  # noqa: F401
